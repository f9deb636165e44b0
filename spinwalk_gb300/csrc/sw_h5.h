// Minimal HDF5 subset (sw_h5.cpp): whole datasets of the root group, uint8 / float / double.
#pragma once
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace sw {
namespace h5 {

enum Type { kU8 = 0, kF32 = 1, kF64 = 2 };

struct Dataset {
    std::vector<uint64_t> dims;
    Type type = kF32;
    std::vector<char> data;     // little-endian, row-major
};

bool read(const std::string &file, const std::string &name, Dataset &out, std::string &err);
bool exists(const std::string &file, const std::string &name);
bool list(const std::string &file, std::vector<std::string> &names, std::string &err);
bool write(const std::string &file, const std::vector<std::pair<std::string, Dataset>> &sets,
           std::string &err);

}  // namespace h5
}  // namespace sw
