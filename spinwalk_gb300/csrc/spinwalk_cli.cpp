// `spinwalk` command-line host: the `sim` subcommand of SpinWalk's CLI (src/spinwalk.cpp:53-56,
// 130-135) on top of libspinwalk_gpu.
//
//   spinwalk sim -c cfg1.ini [cfg2.ini ...] [-d device]
//   spinwalk --version | -g/--gpu_info
//
// Each config runs like monte_carlo::run (sw_run_config). The reference's `-p/--use_cpu` CPU
// path does not exist here: this build runs the GPU kernels only, and says so.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "spinwalk_gpu.h"

static int usage() {
    std::fprintf(stderr,
                 "usage: spinwalk sim -c <config.ini> [more.ini ...] [-d <device>]\n"
                 "       spinwalk --version | --gpu_info\n");
    return 1;
}

int main(int argc, char **argv) {
    if (argc < 2) return usage();
    const std::string cmd = argv[1];
    if (cmd == "-v" || cmd == "--version") {
        std::printf("spinwalk (GB300 sim path) ABI %d\n", sw_abi_version());
        return 0;
    }
    if (cmd == "-g" || cmd == "--gpu_info") {
        int n = 0;
        sw_device_count(&n);
        std::printf("GPUs: %d\n", n);
        return n > 0 ? 0 : 1;
    }
    if (cmd != "sim") return usage();
    std::vector<std::string> configs;
    int device = 0;
    for (int i = 2; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "-c" || a == "--configs") {
            while (i + 1 < argc && argv[i + 1][0] != '-') configs.push_back(argv[++i]);
        } else if ((a == "-d" || a == "--device") && i + 1 < argc) {
            device = std::atoi(argv[++i]);
        } else if (a == "-p" || a == "--use_cpu") {
            std::fprintf(stderr, "spinwalk: this build has no CPU path; it runs on the GPU only\n");
            return 1;
        } else {
            return usage();
        }
    }
    if (configs.empty()) return usage();
    for (const auto &c : configs) {
        if (sw_run_config(c.c_str(), device) != SW_OK) {
            std::fprintf(stderr, "spinwalk: simulation failed for %s: %s\n", c.c_str(), sw_last_error());
            return 1;
        }
    }
    return 0;
}
