// `spinwalk` command-line host: the `sim` subcommand of SpinWalk's CLI (src/spinwalk.cpp:49-56,
// 100-135) on top of libspinwalk_gpu.
//
//   spinwalk [-l|--log <file>] sim -c|--configs cfg1.ini [cfg2.ini ...] [-d|--device <id>]
//   spinwalk -v|--version | -g|--gpu_info
//
// Each config runs like monte_carlo::run (sw_run_config), in order; the first failure stops the
// run with exit code 1, as sim::handler::execute does (src/sim/handler.cu:7-15). As in the
// reference, a log file (default log_spinwalk.txt in the working directory) is appended with
// "[time stamp] [severity]: message" lines, one per config started, finished or failed.
// Long options also take the --name=value form. The reference's `-p/--use_cpu` CPU path does
// not exist here: this build runs the GPU kernels only, and says so.
#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "spinwalk_gpu.h"

namespace {

int usage() {
    std::fprintf(stderr,
                 "usage: spinwalk [-l <log file>] sim -c <config.ini> [more.ini ...] [-d <device>]\n"
                 "       spinwalk --version | --gpu_info\n");
    return 1;
}

// Appends one line in the reference's log format ("[%TimeStamp%] [%Severity%]: %Message%").
void log_line(const std::string &path, const char *severity, const std::string &msg) {
    FILE *f = std::fopen(path.c_str(), "a");
    if (!f) return;
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    struct tm t;
    localtime_r(&tv.tv_sec, &t);
    char stamp[64];
    std::strftime(stamp, sizeof stamp, "%Y-%b-%d %H:%M:%S", &t);
    std::fprintf(f, "[%s.%06ld] [%s]: %s\n", stamp, (long)tv.tv_usec, severity, msg.c_str());
    std::fclose(f);
}

// "--name=value" -> value for a long option `name`; nullptr if `arg` is not that form.
const char *eq_value(const std::string &arg, const char *name) {
    const size_t n = std::strlen(name);
    if (arg.compare(0, n, name) == 0 && arg.size() > n && arg[n] == '=') return arg.c_str() + n + 1;
    return nullptr;
}

std::string base_name(const std::string &p) {
    const size_t s = p.find_last_of('/');
    return s == std::string::npos ? p : p.substr(s + 1);
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) return usage();
    std::string log_file = "log_spinwalk.txt";
    int i = 1;
    for (; i < argc; i++) {                          // options before the subcommand
        const std::string a = argv[i];
        if (a == "-v" || a == "--version") {
            std::printf("spinwalk (GB300 sim path) ABI %d\n", sw_abi_version());
            return 0;
        }
        if (a == "-g" || a == "--gpu_info") {         // sim::print_device_info
            char info[1024];
            const int rc = sw_device_info(0, info, sizeof info);
            std::printf("%s", info);
            return rc == SW_OK ? 0 : 1;
        }
        if ((a == "-l" || a == "--log") && i + 1 < argc) {
            log_file = argv[++i];
        } else if (const char *v = eq_value(a, "--log")) {
            log_file = v;
        } else {
            break;
        }
    }
    if (i >= argc || std::string(argv[i]) != "sim") return usage();
    std::vector<std::string> configs;
    int device = 0;
    for (i++; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "-c" || a == "--configs") {
            while (i + 1 < argc && argv[i + 1][0] != '-') configs.push_back(argv[++i]);
        } else if (const char *v = eq_value(a, "--configs")) {
            configs.push_back(v);
            while (i + 1 < argc && argv[i + 1][0] != '-') configs.push_back(argv[++i]);
        } else if ((a == "-d" || a == "--device") && i + 1 < argc) {
            device = std::atoi(argv[++i]);
        } else if (const char *v = eq_value(a, "--device")) {
            device = std::atoi(v);
        } else if (a == "-p" || a == "--use_cpu") {
            std::fprintf(stderr, "spinwalk: this build has no CPU path; it runs on the GPU only\n");
            log_line(log_file, "error", "--use_cpu requested: this build runs on the GPU only");
            return 1;
        } else {
            return usage();
        }
    }
    if (configs.empty()) return usage();
    std::printf("Log file location: %s\n", log_file.c_str());
    for (const auto &c : configs) {
        std::printf("<%s>\n", base_name(c).c_str());
        std::fflush(stdout);
        log_line(log_file, "info", "Simulating " + c + " on device " + std::to_string(device));
        if (sw_run_config(c.c_str(), device) != SW_OK) {
            const std::string err = sw_last_error();
            log_line(log_file, "error", c + ": " + err);
            std::fprintf(stderr, "spinwalk: simulation failed for %s: %s\n", c.c_str(), err.c_str());
            std::printf("Simulation failed. See the log file %s, Aborting...!\n", log_file.c_str());
            return 1;
        }
        log_line(log_file, "info", "Finished " + c);
    }
    std::printf("Simulation completed successfully. See the log file\n");
    return 0;
}
