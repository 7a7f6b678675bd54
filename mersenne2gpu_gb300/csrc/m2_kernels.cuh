// m2_kernels.cuh -- kernel parameter blocks and launch wrappers (host-visible).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace m2k {

// Dual-field twiddle as stored on the device (24 bytes, same as m2::Dual).
struct DTw { unsigned long long a, b; unsigned int c, d; };

enum Mode : int { LL = 0, PRP = 1, PRP3 = 2 };

// Status word written by kernels (0 = ok).
enum Status : int { ST_OK = 0, ST_CARRY_RANGE = 1, ST_NORMALIZE = 2, ST_WAIT_TIMEOUT = 4 };

// One independent test for the whole-iteration-in-one-CTA kernel.
struct SmallTest {
    long long* digits;        // n balanced digits (in/out)
    const unsigned char* w61; // n shifts
    const unsigned char* w31;
    const DTw* tw4;           // radix-4 twiddles of this h
    const DTw* tc;            // centre twiddles of this h
    int* status;
    unsigned int p;
    unsigned int iters;
    int ln;
    int mode;
    int span;                 // carry span (digits normalized after a segment carry)
    int carry_threads;        // threads taking part in the segmented carry (0 = one thread, full normalization)
    int gf61_only;            // 1: the GF(P61) residue alone is the convolution word (no CRT)
    int fuse_middle;          // 1: the last forward level, the centre and the first inverse level in one pass
};

// Plan of the three-pass path for one transform length.
struct LargePlan {
    int ln, L, L1, L2;        // log2 n, log2 h, log2 rows, log2 row length
    unsigned int R, B, C, G;  // rows, row length, columns per CTA, column groups
    int span;
    unsigned int p;
    int mode;
    unsigned int mid_tickets;  // fused column kernel: 0 = cooperative (CTA index = group), 1 = groups by arrival ticket
    unsigned int gf61;         // 1: the GF(P61^2)-only layout; each word is the signed GF(P61) residue (no CRT)
    unsigned int mid_barrier;  // cooperative fused column kernel: 1 = all groups publish before any goes on
};

struct LargeBufs {
    long long* digits;        // n
    long long* carries;       // R*G segment carries
    ulonglong2* za;           // h GF(P61^2) coordinates
    uint2* zb;                // h GF(P31^2) coordinates
    const unsigned char* w61;
    const unsigned char* w31;
    const DTw* tw4;
    const DTw* tc;
    int* status;
    unsigned int* flags;      // G epoch flags of the fused column kernel, then its 64-bit ticket counter and
    unsigned long long* ticket;   // its 64-bit phase counter (zero-initialised)
    unsigned long long* phase;
    // per element k (digits 2k, 2k+1): x = the two digits' unweighting rotations mod 61 (bytes 0, 1) and
    // mod 31 (bytes 2, 3), y = their widths (bytes 0, 1); read by the quad-shuffle column passes
    const uint2* aux;
};

constexpr int LARGE_STAGES = 3;
constexpr int STAGE_MID = 3;   // the fused inverse + forward column pass (k_cols_mid_q)

// Throughput of 32x32->64-bit integer multiplies (mul.wide.u32 / mad.wide.u32)
// on every SM: independent chains, returns products per second.
double measure_wide_mul_rate(int device);

// ---- full carry propagation (m2_carry.cu) ----
struct NormSum;
struct NormArgs {
    const long long* digits;          // n signed digit words
    const long long* carries;         // pending segment carries (n / seg of them) or null
    unsigned long long seg;           // digits per segment (a multiple of 8) when carries != null
    unsigned long long n, p;
    int ln;
    unsigned long long* out;          // n canonical digits
    int* status;                      // |= 2 when the state is outside the propagation's range
    NormSum* block_sum;               // scratch (norm_bind_scratch)
    long long* block_cin;
    unsigned int* flags;              // bit 0: the result was all ones (written as zero); bit 1: a digit >= 8 is nonzero
};
size_t norm_scratch_bytes(unsigned long long n);
void norm_bind_scratch(NormArgs& a, void* scratch);
cudaError_t launch_normalize(const NormArgs& a, cudaStream_t s);
// canonical digits -> balanced digits with no pending carries; *bad |= 1 when
// an input digit is not canonical (bad may be null)
cudaError_t launch_balance(const unsigned long long* canon, long long* digits, unsigned long long p, int ln,
                           unsigned long long n, unsigned int* bad, cudaStream_t s);

}  // namespace m2k

// The transform kernels are built twice (m2_field.cuh): M2_DUAL = 1 into
// namespace m2k, M2_DUAL = 0 (GF(P61^2) alone) into m2k_g61.  A kernel build
// sees only its own entry points, so that calls inside it resolve to them.
#ifndef M2_DUAL
#define M2_DUAL 1
#endif
#if M2_DUAL
#define M2K_NS m2k
namespace m2k {
#include "m2_launch.inc"
}  // namespace m2k
#else
#define M2K_NS m2k_g61
#endif
namespace m2k_g61 {
using namespace m2k;
#include "m2_launch.inc"
}  // namespace m2k_g61
