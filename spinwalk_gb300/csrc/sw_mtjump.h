// Jump-ahead of std::mt19937 (host side): the polynomials that let k_seed_jump compute the state
// after discard(z) in a number of steps independent of z.
//
// The reference seeds every spin's two generators with mt19937(seed + spin) and then calls
// discard(seed + spin) on each (src/sim/kernels.cu:82-88): spin s costs seed + s generated words,
// which grows without bound with the seed (a config with SEED = 0 draws a random 32-bit seed,
// simulation_parameters.cuh:233-234). The mt19937 state transition T (one generated word) is
// linear over GF(2) on the 19937-bit state, with characteristic polynomial phi of degree 19937
// (primitive; 135 nonzero terms). For any J, T^J = g(T) with g = x^J mod phi, so
// state_J = sum over k with g_k = 1 of state_k: an XOR of 19937 state windows of the spin's own
// output sequence. This is the polynomial jump-ahead of Haramoto, Matsumoto, Nishimura, Panneton
// and L'Ecuyer, "Efficient jump ahead for F2-linear random number generators" (2008).
#pragma once
#include <cstdint>
#include <vector>

namespace sw {

constexpr int kMtDegree = 19937;
constexpr int kJumpPolyWords = 624;   // 19937 coefficients, bit k of word k / 32

// Exponents of the nonzero terms of phi, ascending (0 first, 19937 last); computed once by the
// Berlekamp-Massey algorithm over GF(2) from 2 x 19937 output bits of std::mt19937.
const std::vector<int> &mt_charpoly_terms();

// For R = R_lo .. R_lo + count - 1: the coefficients of x^(624 R - 1) mod phi, 624 words per R
// (bits >= 19937 zero). 624 R - 1 words after seeding is the state whose window starts one word
// before the R-th regeneration's block (what discard(z) with z in (624 (R-1), 624 R] leaves).
void mt_jump_polys(uint64_t R_lo, uint32_t count, uint32_t *out);

// The state of mt19937(z) after discard(z) computed on the host through the polynomial: the
// 624-word block after the last regeneration and the position in it (tests).
void mt_jump_state_host(uint64_t z, uint32_t *block, uint32_t *pos);

// Regenerations that discard(z) performs right after seeding (as mt_discard_twists).
inline uint64_t mt_regenerations(uint64_t z) { return z == 0 ? 0 : 1 + (z - 1) / 624; }

}  // namespace sw
