// Jump-ahead polynomials of std::mt19937 (see sw_mtjump.h).
//
// Polynomials over GF(2) are bit vectors in 64-bit words, bit k = coefficient of x^k. phi has
// 135 nonzero terms and its second-highest exponent is 19314, 623 below the leading 19937, so a
// reduction folds up to 623 bits at a time: bits [lo, lo + 623) at or above x^19937 are cleared
// and added back at lo - 19937 + d for every lower term x^d of phi, all of which lands below lo.
#include "sw_mtjump.h"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <random>
#include <stdexcept>

namespace sw {
namespace {

constexpr int kW = (2 * kMtDegree + 64) / 64 + 2;   // words of a product before reduction
constexpr int kFold = 623;                            // bits folded per reduction pass

inline bool bit_at(const uint64_t *a, int k) { return (a[k >> 6] >> (k & 63)) & 1u; }

// a ^= src[0 .. nbits) shifted left by `shift` bits (a must hold the shifted range)
void xor_shifted(uint64_t *a, const uint64_t *src, int nbits, int shift) {
    const int nw = (nbits + 63) >> 6, q = shift >> 6, r = shift & 63;
    for (int i = 0; i < nw; i++) {
        uint64_t v = src[i];
        if (i == nw - 1 && (nbits & 63)) v &= (uint64_t(1) << (nbits & 63)) - 1;
        if (r == 0) {
            a[q + i] ^= v;
        } else {
            a[q + i] ^= v << r;
            if (v >> (64 - r)) a[q + i + 1] ^= v >> (64 - r);
        }
    }
}

// bits [lo, lo + n) of a into out (n <= 640)
void extract(const uint64_t *a, int lo, int n, uint64_t *out) {
    const int nw = (n + 63) >> 6, q = lo >> 6, r = lo & 63;
    for (int i = 0; i < nw; i++) {
        uint64_t v = a[q + i] >> r;
        if (r) v |= a[q + i + 1] << (64 - r);
        out[i] = v;
    }
    if (n & 63) out[nw - 1] &= (uint64_t(1) << (n & 63)) - 1;
}

void clear_bits(uint64_t *a, int lo, int hi) {
    for (int k = lo; k < hi; k++) {
        if (!(k & 63) && k + 64 <= hi) {
            a[k >> 6] = 0;
            k += 63;
        } else {
            a[k >> 6] &= ~(uint64_t(1) << (k & 63));
        }
    }
}

int top_bit(const uint64_t *a, int nw) {
    for (int i = nw - 1; i >= 0; i--)
        if (a[i]) return 64 * i + 63 - __builtin_clzll(a[i]);
    return -1;
}

// a <- a mod phi (a holds kW words; its degree may be anything below 64 kW - 64)
void reduce(uint64_t *a, const std::vector<int> &terms) {
    int hi = top_bit(a, kW) + 1;
    uint64_t chunk[11];
    while (hi > kMtDegree) {
        const int lo = std::max(kMtDegree, hi - kFold);
        extract(a, lo, hi - lo, chunk);
        clear_bits(a, lo, hi);
        for (size_t t = 0; t + 1 < terms.size(); t++)        // the terms below x^19937
            xor_shifted(a, chunk, hi - lo, lo - kMtDegree + terms[t]);
        hi = lo;
        while (hi > kMtDegree && !bit_at(a, hi - 1)) hi--;
    }
}

// a <- a^2 mod phi: the square of a GF(2) polynomial spreads its bits to even positions
void square(uint64_t *a, const std::vector<int> &terms) {
    static const auto spread = [] {
        std::vector<uint16_t> t(256);
        for (int v = 0; v < 256; v++) {
            uint16_t s = 0;
            for (int b = 0; b < 8; b++)
                if (v >> b & 1) s |= (uint16_t)(1u << (2 * b));
            t[v] = s;
        }
        return t;
    }();
    const int nw = (kMtDegree + 63) / 64;
    uint64_t out[kW];
    std::memset(out, 0, sizeof(out));
    for (int i = 0; i < nw; i++) {
        const uint64_t v = a[i];
        uint64_t lo = 0, hi = 0;
        for (int b = 0; b < 4; b++) {
            lo |= (uint64_t)spread[(v >> (8 * b)) & 0xff] << (16 * b);
            hi |= (uint64_t)spread[(v >> (32 + 8 * b)) & 0xff] << (16 * b);
        }
        out[2 * i] = lo;
        out[2 * i + 1] = hi;
    }
    std::memcpy(a, out, sizeof(out));
    reduce(a, terms);
}

// a <- a * x^k mod phi (k < 64 * (kW - 313))
void mul_xk(uint64_t *a, int k, const std::vector<int> &terms) {
    uint64_t out[kW];
    std::memset(out, 0, sizeof(out));
    xor_shifted(out, a, kMtDegree, k);
    std::memcpy(a, out, sizeof(out));
    reduce(a, terms);
}

// x^J mod phi
void pow_x(uint64_t J, uint64_t *a, const std::vector<int> &terms) {
    std::memset(a, 0, sizeof(uint64_t) * kW);
    a[0] = 1;
    if (J == 0) return;
    int top = 63 - __builtin_clzll(J);
    // the leading bits form an exponent below 2^14, which x^e reaches without reduction work
    int b = top;
    uint64_t e = 0;
    while (b >= 0 && (e << 1 | ((J >> b) & 1)) < 16384) {
        e = e << 1 | ((J >> b) & 1);
        b--;
    }
    a[0] = 0;
    a[e >> 6] = uint64_t(1) << (e & 63);
    reduce(a, terms);
    for (; b >= 0; b--) {
        square(a, terms);
        if ((J >> b) & 1) mul_xk(a, 1, terms);
    }
}

// Berlekamp-Massey over GF(2) on the low output bit of std::mt19937: returns the exponents of
// the recurrence's characteristic polynomial (the reversed connection polynomial).
std::vector<int> berlekamp_massey_mt() {
    const int N = 2 * kMtDegree;
    std::mt19937 gen;                                  // default seed; any nonzero state works
    std::vector<uint8_t> s(N);
    for (int i = 0; i < N; i++) s[i] = gen() & 1u;
    // r: the sequence reversed and packed, so that s[n - i] for i = 0 .. L is a bit range
    const int RW = N / 64 + 3;
    std::vector<uint64_t> r(RW, 0);
    for (int i = 0; i < N; i++) {
        const int j = N - 1 - i;
        if (s[i]) r[j >> 6] |= uint64_t(1) << (j & 63);
    }
    // C and B have degree <= N; B x^m is added with m <= N, so twice the words hold it
    const int PW = 2 * (N / 64 + 3);
    std::vector<uint64_t> C(PW, 0), B(PW, 0), T(PW);
    C[0] = B[0] = 1;
    int L = 0, m = 1;
    for (int n = 0; n < N; n++) {
        // d = sum_{i=0..L} c_i s[n-i]; s[n-i] is bit (N-1-n+i) of r
        const int off = N - 1 - n;
        uint64_t acc = 0;
        for (int w = 0; w <= L / 64; w++) {
            const int pos = off + 64 * w, q = pos >> 6, sh = pos & 63;
            uint64_t v = r[q] >> sh;
            if (sh && q + 1 < RW) v |= r[q + 1] << (64 - sh);
            uint64_t c = C[w];
            if (w == L / 64 && ((L + 1) & 63)) c &= (uint64_t(1) << ((L + 1) & 63)) - 1;
            acc ^= c & v;
        }
        const int d = __builtin_popcountll(acc) & 1;
        if (!d) {
            m++;
        } else if (2 * L <= n) {
            T = C;
            xor_shifted(C.data(), B.data(), N + 1, m);
            L = n + 1 - L;
            B = T;
            m = 1;
        } else {
            xor_shifted(C.data(), B.data(), N + 1, m);
            m++;
        }
    }
    std::vector<int> terms;
    for (int i = 0; i <= L; i++)
        if ((C[i >> 6] >> (i & 63)) & 1) terms.push_back(L - i);
    std::sort(terms.begin(), terms.end());
    if (L != kMtDegree || terms.front() != 0 || terms.back() != kMtDegree)
        throw std::runtime_error("mt19937 characteristic polynomial: unexpected degree");
    // the fold width relies on a gap of at least 623 below the leading term
    if (terms[terms.size() - 2] > kMtDegree - kFold)
        throw std::runtime_error("mt19937 characteristic polynomial: unexpected second term");
    return terms;
}

}  // namespace

// The state of mt19937(z) after discard(z), on the host, by the jump polynomial: the block after
// the last regeneration and the position in it (libstdc++'s _M_x / _M_p). For tests of the
// polynomials; k_seed_jump does the same on the GPU.
void mt_jump_state_host(uint64_t z, uint32_t *block, uint32_t *pos) {
    const uint64_t R = mt_regenerations(z);
    std::vector<uint32_t> x(kMtDegree + 2 * 624 + 64);
    x[0] = (uint32_t)z;
    for (uint32_t i = 1; i < 624; i++) x[i] = 1812433253u * (x[i - 1] ^ (x[i - 1] >> 30)) + i;
    if (R == 0) {
        std::memcpy(block, x.data(), 624 * 4);
        *pos = 624;
        return;
    }
    auto twist = [](uint32_t a, uint32_t b, uint32_t m) {
        const uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
        return m ^ (y >> 1) ^ ((b & 1u) ? 0x9908b0dfu : 0u);
    };
    for (size_t n = 624; n < x.size(); n++) x[n] = twist(x[n - 624], x[n - 623], x[n - 227]);
    std::vector<uint32_t> g(kJumpPolyWords);
    mt_jump_polys(R, 1, g.data());
    uint32_t h[624] = {};
    for (int k = 0; k < kMtDegree; k++)
        if ((g[k >> 5] >> (k & 31)) & 1u)
            for (int j = 0; j < 624; j++) h[j] ^= x[k + j];
    for (int q = 0; q < 623; q++) block[q] = h[q + 1];
    block[623] = twist(h[0], h[1], h[397]);
    *pos = (uint32_t)(z - 624 * (R - 1));
}

const std::vector<int> &mt_charpoly_terms() {
    static const std::vector<int> terms = berlekamp_massey_mt();
    return terms;
}

void mt_jump_polys(uint64_t R_lo, uint32_t count, uint32_t *out) {
    if (count == 0) return;
    const std::vector<int> &terms = mt_charpoly_terms();
    uint64_t a[kW];
    pow_x(R_lo ? 624 * R_lo - 1 : 0, a, terms);
    for (uint32_t i = 0; i < count; i++) {
        if (i) mul_xk(a, 624, terms);
        uint32_t *o = out + (size_t)i * kJumpPolyWords;
        for (int w = 0; w < kJumpPolyWords; w++)
            o[w] = (uint32_t)(a[w >> 1] >> (32 * (w & 1)));
    }
}

}  // namespace sw

extern "C" int sw_debug_mt_jump(uint64_t z, uint32_t *block, uint32_t *pos) {
    if (!block || !pos) return -1;                        // SW_ERR_INVALID
    try {
        sw::mt_jump_state_host(z, block, pos);
    } catch (const std::exception &) {
        return -1;
    }
    return 0;
}
