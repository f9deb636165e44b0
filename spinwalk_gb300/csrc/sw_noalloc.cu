// sw_sim_device_noalloc: the device-buffer simulation entry point for callers that must not
// allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- a host process whose device
// memory is fully reserved up front by a pool or by another framework's allocator, a real-time
// loop that cannot afford cudaMalloc's implicit device-wide synchronisation, or an embedding
// application whose rules forbid a library from allocating behind its back. They pass their
// own inputs and outputs; everything else the walk needs (generator state, per-spin state,
// parameter tables, the logf correction bitmap) lives in one static device array of fixed size,
// SW_NOALLOC_SCRATCH_BYTES, that every GPU which loads this module keeps until the process
// exits.
//
// It runs the same kernels as sw_sim_device, in FP32 precision, and writes the same outputs.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "spinwalk_gpu.h"
#include "sw_api_internal.h"
#include "sw_host.h"
#include "sw_kernels.h"

// The static scratch region (the only device memory this entry point uses besides the caller's
// buffers). Layout: [0, 1 KiB) logf reduction table | [1 KiB, ~48 MiB) logf bitmap |
// per-call workspace (packed phantom, tables, per-spin state, generator state).
static __device__ __align__(256) unsigned char g_noalloc_scratch[SW_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr size_t kBitmapOffset = 1024;
constexpr int kMaxDevices = 64;

struct StaticRegion {
    std::mutex mu;
    char *base = nullptr;        // device address of g_noalloc_scratch on this device
    size_t work_offset = 0;      // start of the per-call workspace
};
StaticRegion g_region[kMaxDevices];

// Once per device, with that device current: resolve the array's device address (in host code
// the symbol is only a stand-in) and write the logf tables into its head.
int setup(StaticRegion &r) {
    if (r.base) return SW_OK;
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
        cudaGetLastError();
        return sw::api::fail(SW_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") +
                                              cudaGetErrorString(e));
    }
    const sw::LogfExceptions &ex = sw::logf_exceptions();
    if (ex.wide != 0)
        return sw::api::fail(SW_ERR_INVALID, "host logf does not match the device candidate rule");
    const size_t bitmap_bytes = ex.bitmap.size() * sizeof(uint32_t);
    char *base = static_cast<char *>(ptr);
    e = cudaMemcpy(base, sw::logf_reduction_table(), 192 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(base + kBitmapOffset, ex.bitmap.data(), bitmap_bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return sw::api::fail(SW_ERR_CUDA, std::string("logf table upload: ") + cudaGetErrorString(e));
    }
    r.work_offset = (kBitmapOffset + bitmap_bytes + 255) & ~size_t(255);
    r.base = base;
    return SW_OK;
}

}  // namespace

extern "C" int sw_sim_device_noalloc(const sw_params *p, const sw_sequence *q,
                                     const float *d_FieldMap, const uint8_t *d_Mask,
                                     const float *d_M0, const float *d_XYZ0, float *d_M1,
                                     float *d_XYZ1, uint8_t *d_T, int32_t *d_status,
                                     void *stream) {
    using namespace sw::api;
    int rc = check_args(p, q);
    if (rc) return rc;
    if (p->n_spins == 0) return SW_OK;
    if (!d_Mask || !d_M0 || !d_XYZ0 || !d_XYZ1 || (q->n_TE && (!d_M1 || !d_T)))
        return fail(SW_ERR_INVALID, "null device buffer");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(SW_ERR_CUDA, "no current CUDA device");
    }
    StaticRegion &R = g_region[dev];
    std::lock_guard<std::mutex> lk(R.mu);
    rc = setup(R);
    if (rc) return rc;

    TableImage im;
    build_tables(p, q, im);
    if (!im.complete()) return fail(SW_ERR_INVALID, "internal error: incomplete parameter tables");
    const size_t need = layout(nullptr, p->n_spins, p->matrix_length, im.bytes.size(), false).bytes;
    const size_t avail = SW_NOALLOC_SCRATCH_BYTES - R.work_offset;
    if (need > avail)
        return fail(SW_ERR_NOMEM,
                    "sw_sim_device_noalloc: this problem needs " + std::to_string(need >> 20) +
                        " MiB of scratch (about 8.5 KiB per spin + 8 B per voxel) but the static "
                        "array has " + std::to_string(avail >> 20) + " MiB left after the logf "
                        "table; use fewer spins per call or sw_sim_device");
    const Layout L = layout(R.base + R.work_offset, p->n_spins, p->matrix_length,
                            im.bytes.size(), false);
    cudaStream_t st = (cudaStream_t)stream;
    // On an error the call first waits for what it already queued on `stream`, so that no
    // kernel of a failed call still writes the shared array when the next call takes it over.
#define NA_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            cudaGetLastError();                                                            \
            cudaStreamSynchronize(st);                                                     \
            cudaGetLastError();                                                            \
            return fail(SW_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
        }                                                                                  \
    } while (0)
    // pageable source: the copy is staged before cudaMemcpyAsync returns
    NA_CUDA(cudaMemcpyAsync(L.tables, im.bytes.data(), im.bytes.size(), cudaMemcpyHostToDevice, st));
    const sw::DevParams P = dev_params(p, q);
    const sw::DevTables Tb = dev_tables(im, L.tables);
    const sw::LogfTables LT{reinterpret_cast<const float *>(R.base),
                            reinterpret_cast<const uint32_t *>(R.base + kBitmapOffset)};
    const sw::Outputs O{d_M1, nullptr, d_XYZ1, d_T, d_status};

    // the counters the previous call left behind must start at zero
    NA_CUDA(cudaMemsetAsync(L.active, 0, 2 * sizeof(uint32_t), st));
    NA_CUDA(sw::launch_pack(d_Mask, p->fieldmap_exist ? d_FieldMap : nullptr, L.vox,
                            p->matrix_length, p->n_substrate, L.active + 1, st));
    NA_CUDA(sw::launch_seed(P, L.G, st));
    NA_CUDA(sw::launch_init(P, Tb, L.vox, d_M0, d_XYZ0, L.S, O, false, st));
    uint32_t h = 0;
    NA_CUDA(cudaMemcpyAsync(&h, L.active + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    if (h != 0) return fail(SW_ERR_INVALID, "the mask holds substrate labels >= n_substrate");
    const uint64_t steps = (uint64_t)p->n_timepoints * (uint64_t)(p->n_dummy_scan + 1);
    const uint64_t max_rounds = 64 + steps * (p->max_iterations + 2);
    const sw_tuning tu = current_tuning();
    for (uint64_t round = 0;; round++) {
        if (round >= max_rounds) {          // every round was waited for: nothing in flight
            return fail(SW_ERR_TIMEOUT, "walk did not finish");
        }
        NA_CUDA(cudaMemsetAsync(L.active, 0, sizeof(uint32_t), st));
        NA_CUDA(sw::launch_refill(P, L.G, L.S, LT, st));
        if (tu.resort_interval && round % tu.resort_interval == 0)
            NA_CUDA(sw::launch_order(P, L.S, L.Q, 0, P.n_spins, st));
        NA_CUDA(sw::launch_walk_range(SW_PREC_FP32, false, P, Tb, L.vox, L.S, L.G, O, L.active, 0,
                                      P.n_spins, st, tu.resort_interval ? L.Q.order : nullptr,
                                      (int)tu.walk_block));
        NA_CUDA(cudaMemcpyAsync(&h, L.active, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        NA_CUDA(cudaStreamSynchronize(st));
        if (h == 0) break;
    }
#undef NA_CUDA
    return SW_OK;
}
