// Checks sw::h5::convert_value (sw_h5.h), the conversion sw_run_config applies to phantom and
// start-file datasets stored in other types than the reference reads (libhdf5's rules: integers
// saturate, floats truncate toward zero, NaN -> 0). Prints "ok <checks>" or the first failure.
#include <cmath>
#include <cstdio>
#include <limits>

#include "sw_h5.h"

using sw::h5::convert_value;

static int checks = 0, bad = 0;

template <typename T, typename S>
void expect(S v, T want, const char *what) {
    const T got = convert_value<T>(v);
    checks++;
    if (!(got == want || (got != got && want != want))) {
        bad++;
        std::printf("FAIL %s: got %.17g want %.17g\n", what, (double)got, (double)want);
    }
}

int main() {
    const double nan = std::nan("");
    // masks: MATLAB writes int8, h5py may write int64 or double
    expect<uint8_t, int8_t>(3, 3, "int8 3 -> u8");
    expect<uint8_t, int8_t>(-1, 0, "int8 -1 -> u8 saturates at 0");
    expect<uint8_t, int8_t>(127, 127, "int8 127 -> u8");
    expect<uint8_t, int64_t>(300, 255, "int64 300 -> u8 saturates at 255");
    expect<uint8_t, int64_t>(-5, 0, "int64 -5 -> u8");
    expect<uint8_t, uint64_t>(~0ull, 255, "uint64 max -> u8");
    expect<uint8_t, uint16_t>(200, 200, "uint16 200 -> u8");
    expect<uint8_t, double>(2.0, 2, "double 2 -> u8");
    expect<uint8_t, double>(2.9, 2, "double 2.9 -> u8 truncates");
    expect<uint8_t, double>(-0.5, 0, "double -0.5 -> u8");
    expect<uint8_t, double>(1e9, 255, "double 1e9 -> u8");
    expect<uint8_t, double>(nan, 0, "double NaN -> u8");
    expect<uint8_t, float>(14.99f, 14, "float 14.99 -> u8");
    expect<int8_t, int32_t>(-200, -128, "int32 -200 -> i8 saturates");
    expect<int8_t, uint32_t>(4000000000u, 127, "uint32 4e9 -> i8 saturates");
    expect<int8_t, double>(-3.7, -3, "double -3.7 -> i8 truncates toward zero");
    // fieldmap / fov / XYZ / M read as float
    expect<float, double>(0.1, (float)0.1, "double 0.1 -> float rounds to nearest");
    expect<float, double>(1e-4, (float)1e-4, "double fov -> float");
    expect<float, int16_t>(-7, -7.0f, "int16 -> float");
    expect<float, uint8_t>(200, 200.0f, "u8 -> float");
    expect<float, float>(1.5f, 1.5f, "float -> float");
    if (bad) return 1;
    std::printf("ok %d\n", checks);
    return 0;
}
