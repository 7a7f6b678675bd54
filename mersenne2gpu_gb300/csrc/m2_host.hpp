// m2_host.hpp -- host-side tables and state conversion for the GB300 engine.
//
// Exponent -> transform size, digit widths and IBDWT shift weights follow the
// reference definitions (mersenne2_gpu.cpp:286-293, 3921-3944) because they
// define the residue's digit layout, which must be identical for the state to
// be a drop-in.  The transform itself (generator, twiddle tables, step plan)
// is this engine's own.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace m2 {

using u64 = uint64_t;
using u32 = uint32_t;
using i64 = int64_t;

constexpr u64 P61 = (u64(1) << 61) - 1;
constexpr u32 P31 = (u32(1) << 31) - 1;

// Dual-field element as stored in the twiddle tables: GF(P61^2) pair + GF(P31^2) pair.
struct alignas(8) Dual {
    u64 a, b;   // GF(P61^2): a + b i
    u32 c, d;   // GF(P31^2): c + d i
};
static_assert(sizeof(Dual) == 24, "Dual must be 24 bytes");

// Smallest ln >= 3 with ln + 2((p >> ln) + 1) < bound: 92 for the two fields
// (mersenne2_gpu.cpp:286-293), 61 for GF(P61^2) alone
// (gf61_ntt_prp_opencl_inplace_nobitrev_fused.cpp:124-132).
int transform_log2(u64 p, int bound = 92);

struct Layout {
    u32 p = 0;
    int ln = 0;            // log2 n
    u64 n = 0, h = 0;      // real digits, complex elements
    u32 q = 0;             // narrow digit width p >> ln
    std::vector<uint8_t> width;   // n digit widths, q or q+1
    std::vector<uint8_t> w61;     // n shifts mod 61
    std::vector<uint8_t> w31;     // n shifts mod 31
    std::vector<u64> bitpos;      // n+1 bit positions ceil(p j / n)
};
Layout make_layout(u32 p, int bound = 92);

// Roots of unity of this engine: g61 of order 2^62 in GF(P61^2) and g31 of
// order 2^32 in GF(P31^2), chosen so that the order-4 root is +i.
Dual root_of_unity(u64 order);       // primitive root of the given power-of-two order

// Twiddle tables for the in-place decimation-in-frequency transform of
// length h with per-block twiddles (natural order in, bit-reversed out):
//   tw4[3*(S+j) + a-1] = r^a, r = w_{4S}^{br_S(j)}, for every radix-4 step with
//                        S blocks before the step (S = 1, 4, 16, ...)
//   tc[j]              = w_h^{br_{h/2}(j)}, j < h/2: the centre twiddle of
//                        position 2j; also the radix-2 step's twiddle when
//                        log2 h is odd.
struct Twiddles {
    std::vector<Dual> tw4;   // 3 * (max S of a radix-4 step) * 2 entries
    std::vector<Dual> tc;    // h/2 entries
};
Twiddles make_twiddles(u64 h);

// Bound-driven number of digits through which an incoming segment carry is
// propagated before its remainder is added to the next digit (see the .cpp).
int carry_span(const Layout& L);

// ---- state conversion (exact, host side) ----
// Balanced device state: digits d_j (|d_j| <~ 2^(w_j-1)) and optional pending
// carries carry[s] that belong at bit position bitpos[seg_start[s+1]] (cyclic).
// Returns canonical digits in [0, 2^w_j), all-ones (== M_p) mapped to zero.
std::vector<u64> canonical_digits(const Layout& L, const std::vector<i64>& d,
                                  const std::vector<i64>& carry, u64 seg_digits);
// Any n unsigned digit words -> canonical digits of the residue they denote.
std::vector<u64> canonical_from_unsigned(const Layout& L, const u64* d);
// Canonical (or any non-negative) digits -> balanced digits of the same residue.
std::vector<i64> balanced_digits(const Layout& L, const std::vector<u64>& canon);
// Small integer -> canonical digits.
std::vector<u64> digits_of_small(const Layout& L, u64 x);
u64 res64_of(const Layout& L, const std::vector<u64>& canon);
// Value of canonical digits is exactly `v` (a small integer)?
bool equals_small(const Layout& L, const std::vector<u64>& canon, u64 v);

}  // namespace m2
