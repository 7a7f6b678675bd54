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
};

size_t small_smem_bytes(unsigned int h, int threads);
int small_threads_for(unsigned int h);
// iters_override != 0 replaces every test's iteration count for this launch;
// fuse selects the kernel variant with the fused transform middle (every test
// of the launch must have fuse_middle equal to it)
cudaError_t launch_small(const SmallTest* d_tests, int ntests, unsigned int h, int threads, unsigned int iters_override,
                         cudaStream_t s, bool fuse = false);
// persistent grid: CTAs take test indices from *d_queue (zeroed by the caller)
cudaError_t launch_small_persistent(const SmallTest* d_tests, int ntests, unsigned int h, int threads, int* d_queue,
                                    int grid, cudaStream_t s, bool fuse = false);
int small_ctas_per_sm(unsigned int h, int threads, bool fuse = false);

size_t large_smem_cols(const LargePlan& P);
size_t large_smem_rows(const LargePlan& P);
cudaError_t large_setup(const LargePlan& P);   // sets max dynamic smem attributes
cudaError_t launch_large_iteration(const LargePlan& P, const LargeBufs& b, cudaStream_t s);
constexpr int LARGE_STAGES = 3;
constexpr int STAGE_MID = 3;   // the fused inverse + forward column pass (k_cols_mid_q)
// k squarings: fwd, rows, (mid, rows) x (k - 1), inv when fused, else k x (fwd, rows, inv)
cudaError_t launch_large_run(const LargePlan& P, const LargeBufs& b, unsigned k, bool fused, cudaStream_t s);
// quad-shuffle row pass (m2_rows.cu), used for row lengths 1024 and 2048
bool rows_q_supported(const LargePlan& P);
cudaError_t rows_q_setup(const LargePlan& P);
cudaError_t launch_rows_q(const LargePlan& P, const LargeBufs& b, cudaStream_t s);
// quad-shuffle column passes (m2_cols.cu), used for R = 1024 rows and C = 4
bool cols_q_supported(const LargePlan& P);
cudaError_t cols_q_setup(const LargePlan& P);
cudaError_t launch_cols_q(const LargePlan& P, const LargeBufs& b, bool inverse, cudaStream_t s);
bool cols_mid_supported(const LargePlan& P);     // the fused column kernel serves this plan
bool cols_mid_cooperative(const LargePlan& P);   // ... with all G CTAs co-resident (cooperative launch)
cudaError_t launch_cols_mid(const LargePlan& P, const LargeBufs& b, cudaStream_t s);
cudaError_t launch_large_stage(const LargePlan& P, const LargeBufs& b, int stage, cudaStream_t s);
const char* large_stage_name(int stage);
unsigned long long large_stage_bytes(const LargePlan& P, int stage);

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
