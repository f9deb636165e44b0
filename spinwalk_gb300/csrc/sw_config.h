// Parsed simulation config (sw_config.cpp): the reference's config_reader result.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "spinwalk_gpu.h"

namespace sw {

struct Config {
    sw_params p;                                  // parameters before parameters::prepare
    std::vector<double> diffusivity;              // m^2/s (prepare turns it into step std-devs)
    std::vector<float> T1_ms, T2_ms, pXY, RF_FA_deg, RF_PH_deg, dephasing_deg;
    std::vector<float> gradientX_mTm, gradientY_mTm, gradientZ_mTm, scales;
    std::vector<int32_t> TE_us, RF_us, dephasing_us, gradient_us;   // time points after read
    std::map<std::string, std::vector<std::string>> files;         // PHANTOM, XYZ0, M0
    std::vector<std::string> outputs;
    std::string seq_name, output_dir;
    int scale_type = 0;                           // 0 FoV, 1 gradient, 2 phase cycling
    Config();
};

// read (with PARENT_CONFIG) + check + timing_scale; SW_OK or SW_ERR_CONFIG with `err`.
int config_read(const std::string &path, Config &c, std::string &err);
int config_dump(const Config &c, const std::string &out);

}  // namespace sw
