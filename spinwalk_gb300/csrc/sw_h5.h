// Minimal HDF5 subset (sw_h5.cpp): whole datasets of the root group; little-endian integers of
// 1, 2, 4 or 8 bytes (signed or unsigned), float and double.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace sw {
namespace h5 {

// The codes are those of sw_h5_read / sw_h5_write in the C ABI.
enum Type { kU8 = 0, kF32 = 1, kF64 = 2, kI8 = 3, kU16 = 4, kI16 = 5, kU32 = 6, kI32 = 7,
            kU64 = 8, kI64 = 9 };

inline bool valid_type(int t) { return t >= kU8 && t <= kI64; }
inline bool is_float(Type t) { return t == kF32 || t == kF64; }
inline bool is_signed_int(Type t) { return t == kI8 || t == kI16 || t == kI32 || t == kI64; }
inline size_t type_size(Type t) {
    switch (t) {
    case kU8: case kI8: return 1;
    case kU16: case kI16: return 2;
    case kF32: case kU32: case kI32: return 4;
    default: return 8;
    }
}

struct Dataset {
    std::vector<uint64_t> dims;
    Type type = kF32;
    std::vector<char> data;     // little-endian, row-major
};

// The dataset `name` of the root group; with_data = false fills only dims and type.
bool read(const std::string &file, const std::string &name, Dataset &out, std::string &err,
          bool with_data = true);
bool exists(const std::string &file, const std::string &name);
bool list(const std::string &file, std::vector<std::string> &names, std::string &err);
bool write(const std::string &file, const std::vector<std::pair<std::string, Dataset>> &sets,
           std::string &err);

// One stored value converted to the type the reference reads it as (HighFive hands libhdf5 the
// memory type, and libhdf5 converts): to an integer type, values outside its range saturate,
// floats truncate toward zero and NaN becomes 0; to float or double, the nearest value.
template <typename T, typename S>
T convert_value(S v) {
    if constexpr (std::is_integral_v<T>) {
        if constexpr (std::is_floating_point_v<S>) {
            if (v != v) return T(0);
            if (v <= (S)std::numeric_limits<T>::min()) return std::numeric_limits<T>::min();
            if (v >= (S)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
            return (T)v;
        } else {
            using W = std::conditional_t<std::is_signed_v<S>, int64_t, uint64_t>;
            const W w = (W)v;
            if constexpr (std::is_signed_v<S>)
                if (w < 0 && !std::is_signed_v<T>) return T(0);
            if constexpr (std::is_signed_v<S> && std::is_signed_v<T>)
                if (w < (W)std::numeric_limits<T>::min()) return std::numeric_limits<T>::min();
            if (w > 0 && (uint64_t)w > (uint64_t)std::numeric_limits<T>::max())
                return std::numeric_limits<T>::max();
            return (T)w;
        }
    } else {
        return (T)v;
    }
}

template <typename T, typename S>
void convert_all(const Dataset &d, uint64_t n, std::vector<T> &out) {
    for (uint64_t i = 0; i < n; i++) {
        S v;
        std::memcpy(&v, d.data.data() + i * sizeof(S), sizeof(S));
        out[i] = convert_value<T>(v);
    }
}

// A whole dataset as T, whatever integer or floating type the file stores it in.
template <typename T>
bool read_as(const std::string &file, const char *name, std::vector<T> &out,
             std::vector<uint64_t> *dims, std::string &err) {
    Dataset d;
    if (!read(file, name, d, err)) return false;
    uint64_t n = 1;
    for (uint64_t x : d.dims) n *= x;
    out.resize(n);
    switch (d.type) {
    case kU8: convert_all<T, uint8_t>(d, n, out); break;
    case kI8: convert_all<T, int8_t>(d, n, out); break;
    case kU16: convert_all<T, uint16_t>(d, n, out); break;
    case kI16: convert_all<T, int16_t>(d, n, out); break;
    case kU32: convert_all<T, uint32_t>(d, n, out); break;
    case kI32: convert_all<T, int32_t>(d, n, out); break;
    case kU64: convert_all<T, uint64_t>(d, n, out); break;
    case kI64: convert_all<T, int64_t>(d, n, out); break;
    case kF32: convert_all<T, float>(d, n, out); break;
    case kF64: convert_all<T, double>(d, n, out); break;
    }
    if (dims) *dims = d.dims;
    return true;
}

}  // namespace h5
}  // namespace sw
