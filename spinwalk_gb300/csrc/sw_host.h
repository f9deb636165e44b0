// Host-side helpers of libspinwalk_gpu (sw_host.cpp).
#pragma once
#include <cstdint>
#include <vector>

#include "spinwalk_gpu.h"
#include "sw_types.h"

namespace sw {

struct LogfExceptions {
    std::vector<uint32_t> bitmap;  // [kBitmapWords]: 1 where the host logf != candidate
    uint64_t count = 0;            // inputs marked
    uint64_t wide = 0;             // marked inputs the neighbour rule does not fix (must be 0)
};

const float *logf_reduction_table();            // 64 x {invc, Lhi, Llo}
const LogfExceptions &logf_exceptions();        // built on first use

RfOp make_rf_op(float s, float c, double fa_deg, float ph, int32_t tp);
void build_scan_rf(const sw_params *p, const sw_sequence *q, std::vector<RfOp> &out);
void build_rf(const sw_params *p, const sw_sequence *q, std::vector<RfOp> &out);

}  // namespace sw
