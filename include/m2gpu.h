/*
 * m2gpu.h -- C ABI of the GB300 Lucas-Lehmer / PRP engine (libm2gpu.so).
 *
 * The reference (cherubrock-seb/mersenne2GPU) is one executable: main() owns
 * the OpenCL context, the device buffers z / w / iw / digit_width / blocks /
 * states / carry (mersenne2_gpu.cpp:4010-4028), enqueues an iteration plan p
 * (PRP) or p-2 (LL) times (mersenne2_gpu.cpp:4812-4822) and reads z back once
 * to decide (mersenne2_gpu.cpp:4855-4882).  There is no plugin or FFI API; the
 * entry points below are what its per-iteration contract becomes as a library.
 * The mersenne2 CLI of this project (mersenne2gpu_gb300/csrc/mersenne2_cli.cpp)
 * keeps the reference's command line and output on top of them.
 *
 * Conventions: every function returns 0 or a negative M2_E* code and never
 * exits or traps; device waits are bounded.  A context owns all device memory
 * it uses, the caller owns host buffers.  Calls on one context are not
 * thread-safe; different contexts are independent.  Digits are the residue's
 * n words of width q or q+1 bits (q = p >> log2 n), least significant first,
 * each in [0, 2^width): the same layout as the reference's z[k].s0 / z[k].s1
 * after its carry (mersenne2_gpu.cpp:2116, 3400-3410).
 */
#ifndef M2GPU_H
#define M2GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* test modes: LL and PRP as in mersenne2_gpu.cpp:3454-3462 (TestMode);
 * PRP3 (x <- 3 x^2, p-1 steps, prime iff 3) as in the GF61 prototype
 * gf61_ntt_prp_opencl_inplace_nobitrev_fused.cpp:508-531. */
enum { M2_MODE_LL = 0, M2_MODE_PRP = 1, M2_MODE_PRP3 = 2 };

/* execution path selection (0 = automatic) */
enum { M2_PATH_AUTO = 0, M2_PATH_SMALL = 1, M2_PATH_LARGE = 2 };

/* fields of the transform: GF(P61^2) x GF(P31^2) recombined by CRT (the
 * reference engine, default), or GF(P61^2) alone with the GF61 prototype's
 * size rule ln + 2((p >> ln) + 1) < 61
 * (gf61_ntt_prp_opencl_inplace_nobitrev_fused.cpp:124-132): up to twice the
 * digits, of up to half the width.  Every word of the convolution is then the
 * signed GF(P61) residue, with no CRT; results are the same residues, in that
 * layout's digits.  Both paths and every transform size serve it. */
enum { M2_FIELDS_DUAL = 0, M2_FIELDS_GF61 = 1 };

enum {
    M2_OK = 0,
    M2_EINVAL = -1,       /* bad argument (reference: usage error, exit 1, mersenne2_gpu.cpp:3618-3716) */
    M2_ENOMEM = -2,       /* device allocation failed */
    M2_ECUDA = -3,        /* CUDA runtime error (reference: check() -> exit(1), mersenne2_gpu.cpp:3078-3083) */
    M2_ETIMEOUT = -4,     /* a bounded device wait gave up */
    M2_ESTATE = -5,       /* a kernel reported an out-of-range carry / normalization failure */
    M2_EUNSUPPORTED = -6, /* exponent or option outside what this build supports */
    M2_ECHECK = -7        /* the error check found a wrong state; the context was reset (m2_gec_check) */
};

typedef struct m2_ctx m2_ctx;

/* Options; zero-initialise and set what you need.  The -W / -B knobs of the
 * reference (mersenne2_gpu.cpp:3668-3680) are accepted: wg is the threads per
 * CTA hint, carry_pairs the carry segment size hint (pairs of digits: on the
 * one-CTA path n / (2 carry_pairs) segments, rounded to a power of two and
 * kept within the threads and the carry span; on the three-pass path the
 * columns per CTA). */
typedef struct {
    int device;             /* CUDA device ordinal (reference -d, mersenne2_gpu.cpp:3651-3656) */
    uint32_t wg;            /* -W: threads per CTA hint (0 = auto) */
    uint32_t carry_pairs;   /* -B: carry segment length hint in digit pairs (0 = auto) */
    int path;               /* M2_PATH_* */
    void* stream;           /* cudaStream_t to run on (NULL = the context creates one) */
    int fields;             /* M2_FIELDS_* */
    int fused_middle;       /* one-CTA path: 1 runs the last forward level, the centre square and the first
                               inverse level as one pass (the reference runs them as separate launches,
                               mersenne2_gpu.cpp:4512-4531); 0 = separate passes */
} m2_opts;

typedef struct {
    uint32_t p;
    int mode;
    int ln;                 /* log2 n, the reference's transformsize (mersenne2_gpu.cpp:286-293) */
    uint64_t n;             /* digits */
    uint32_t iteration;     /* squarings applied so far */
    uint32_t total_iters;   /* p-2 (LL), p (PRP), p-1 (PRP3) (mersenne2_gpu.cpp:4780) */
    int path;               /* M2_PATH_SMALL or M2_PATH_LARGE */
    uint32_t rows, row_len, cols_per_cta, span;   /* large-path plan */
    uint64_t device_bytes;  /* device memory held by the context */
    uint32_t fused_cols;    /* 1: the inverse column pass and the next forward one run as one launch */
    int fields;             /* M2_FIELDS_* */
} m2_info_t;

/* Replaces main()'s setup (mersenne2_gpu.cpp:3727-4028): exponent -> transform,
 * tables, buffers, x0 = 4 (LL) / 3 (PRP, PRP3) (mersenne2_gpu.cpp:3908).
 * Transforms up to n = 2^23 digits: p <= 285212671 with both fields,
 * p <= 150994943 with M2_FIELDS_GF61; larger exponents return M2_EUNSUPPORTED
 * (a row of the three-pass plan would no longer fit one CTA's shared memory). */
int m2_create(m2_ctx** out, uint32_t p, int mode, const m2_opts* opts);

/* Replaces k rounds of enqueue_plan(iter_plan); enqueue_plan(post_plan);
 * (mersenne2_gpu.cpp:4812-4822).  Asynchronous on the context's stream. */
int m2_iterate(m2_ctx* ctx, uint32_t k);

/* Replaces clFinish at a report point (mersenne2_gpu.cpp:4788); also reports
 * device-side status (M2_ESTATE). */
int m2_sync(m2_ctx* ctx);

/* Replaces the final clEnqueueReadBuffer of z (mersenne2_gpu.cpp:4855-4863):
 * n canonical digits; the all-ones vector (== M_p) is returned as zero. */
int m2_get_digits(m2_ctx* ctx, uint64_t* out);

/* Sets the state from n digits (any values with digit_j < 2^64; the residue
 * is sum digit_j 2^bitpos_j mod M_p) and the iteration counter (resume). */
int m2_set_digits(m2_ctx* ctx, const uint64_t* digits, uint32_t iteration);

/* Low 64 bits of the canonical residue (the reference prints none; added). */
int m2_res64(m2_ctx* ctx, uint64_t* out);

/* Verdict of the current state: 1 = prime / probable prime, 0 = composite.
 * LL: residue 0 (mersenne2_gpu.cpp:3028-3042); PRP: residue 9
 * (mersenne2_gpu.cpp:3051-3076); PRP3: residue 3. */
int m2_verdict(m2_ctx* ctx, int* is_prime);

int m2_info(m2_ctx* ctx, m2_info_t* info);

/* Releases everything the context owns (mersenne2_gpu.cpp:4884-4958). */
void m2_destroy(m2_ctx* ctx);

/* ---------------- serving engine ----------------
 * No reference counterpart (the reference tests one exponent per process,
 * mersenne2_gpu.cpp:3618-4959).  Continuous batching of independent tests on
 * one GPU: submitted tests wait in a FIFO queue and are admitted while their
 * device memory fits the budget; every m2_srv_step advances each admitted test
 * by up to `quantum` squarings -- tests of one transform size on the one-CTA
 * path share one persistent launch, larger tests run on their own streams, all
 * concurrently -- then retires the finished tests and frees their memory.
 * A test is admitted on an estimate of its device memory and then holds the
 * bytes its context actually allocated (the twiddle tables of a transform size
 * are shared by every test of that size and cached for the process, outside
 * the budget).  Shared one-CTA launches take the batch autotuner's launch
 * shape for their transform size when m2_batch_run has tuned it in this
 * process, else the default shape.
 * Results of a test are identical to running it alone (m2_create/m2_iterate).
 * Times are seconds since m2_srv_create (host steady clock). */
typedef struct m2_server m2_server;

typedef struct {
    uint64_t id;
    uint32_t p;
    int mode;
    uint32_t iters;          /* squarings performed */
    uint64_t res64;
    int is_prime;            /* verdict (meaningful when iters is the full test) */
    int status;              /* M2_OK or an error code */
    uint64_t n;              /* transform length */
    double t_submit, t_admit, t_done;
} m2_srv_result;

typedef struct {
    uint32_t queued, active;
    uint64_t resident_bytes, budget_bytes;
    uint64_t squarings;      /* squarings performed since creation */
    uint64_t completed;
    uint32_t steps, launches;
} m2_srv_stats;

int m2_srv_create(m2_server** out, int device, uint64_t budget_bytes, uint32_t quantum);
/* iters = 0 runs the full test (p-2 / p / p-1 squarings); a test whose device
 * memory alone exceeds the budget is refused with M2_ENOMEM */
int m2_srv_submit(m2_server* s, uint64_t id, uint32_t p, int mode, uint32_t iters);
/* one scheduling round: admit, advance every active test, retire finished ones */
int m2_srv_step(m2_server* s);
/* copies up to max finished results (oldest first) and removes them */
int m2_srv_poll(m2_server* s, m2_srv_result* out, int max, int* n_out);
int m2_srv_stats_get(m2_server* s, m2_srv_stats* st);
/* progress of the admitted (active) tests, in admission order: up to max of
 * them, *n_out = how many were written */
typedef struct {
    uint64_t id;
    uint32_t p;
    uint32_t done;           /* squarings accounted so far */
    uint32_t total;          /* squarings the test will run */
    uint32_t inflight;       /* squarings launched and not yet accounted */
    uint64_t n;              /* transform length */
    uint64_t device_bytes;   /* device memory the test holds */
    double t_submit, t_admit;
} m2_srv_progress;
int m2_srv_active_get(m2_server* s, m2_srv_progress* out, int max, int* n_out);
void m2_srv_destroy(m2_server* s);

/* ---------------- profiling ---------------- */
typedef struct {
    char name[32];
    double ms_per_launch;        /* average device time of one launch */
    uint64_t launches;
    uint64_t bytes_per_launch;   /* algorithmic bytes the stage must read + write */
    uint32_t iters_per_launch;   /* squarings one launch performs */
} m2_stage_time;

/* Runs `iters` squarings with CUDA events around every kernel launch and
 * reports each stage's average device time.  Counterpart of the reference
 * prototype's --profile-kernels (gf61_ntt_prp_opencl_inplace_nobitrev_fused_
 * powonly_blockcarry.cpp:645-698), which sums OpenCL event times per kernel. */
int m2_profile(m2_ctx* ctx, uint32_t iters, m2_stage_time* out, int max_stages, int* n_stages);

/* Kernel launches that m2_iterate(ctx, k) issues. */
uint64_t m2_launches_for(m2_ctx* ctx, uint32_t k);

/* Peak rate of 32x32->64-bit integer products (mad.wide.u32) on a device,
 * products per second: the compute roofline denominator.  No reference
 * counterpart. */
int m2_measure_mul_peak(int device, double* products_per_s);

/* ---------------- squaring without device allocation ----------------
 * No counterpart in the reference.  For callers that may not call cudaMalloc
 * (a framework that owns all device memory through its own pool, or a
 * latency-critical path where an allocation could synchronise the device):
 * advances the residue held in `digits` -- n signed 64-bit words in DEVICE
 * memory, value sum digits[j] 2^bitpos_j mod 2^p - 1, |digits[j]| < 2^width_j
 * (canonical digits qualify) -- by `iters` squarings of `mode` in place, on
 * `stream` (NULL = the legacy default stream) of the current device, and
 * returns when they are done.  Output digits represent the new residue with
 * |digits[j]| <= 2^(width_j - 1) + 8 (not canonical: one carry pass with
 * wrap-around, on the host or the device, makes them canonical).
 * All scratch (element arrays, carries, tables: at most 8 MiB) is one static
 * device array that every GPU loading the library holds until exit; the
 * transform must satisfy 128 <= n <= 2^18 (2689 <= p <= 9437179), larger or
 * smaller exponents return M2_EUNSUPPORTED.  Every call shares that array:
 * calls whose work overlaps on the GPU race.  The first call on a device looks
 * up the array's device address. */
int m2_square_noalloc(uint32_t p, int mode, int64_t* digits, uint32_t iters, void* stream);

/* ---------------- full carry propagation ----------------
 * Replaces the reference's block carry with its serial drain, whose carry out
 * of the top digit re-enters digit 0 (mersenne2_gpu.cpp:2097-2123, 2922-3004).
 * Device pointers, on `stream` of the current device; returns when done.
 * digits: n signed words of exponent p's layout; seg_carries (may be NULL):
 * n / seg_digits words, carry s entering at digit ((s + 1) seg_digits) mod n
 * (seg_digits a multiple of 8 dividing n).  out: the n canonical digits of
 * sum digits_j 2^bitpos_j + sum carry_s 2^bitpos_((s+1) seg) mod 2^p - 1, each
 * in [0, 2^width_j), the all-ones vector (== M_p) written as zero.  The
 * propagation is a parallel carry-lookahead whose range covers every state the
 * engine produces; a state outside it (carries between 8-digit chunks of
 * 2^width or more) returns M2_ESTATE.  Transforms of n <= 64 digits are
 * propagated sequentially and accept any input.  m2_get_digits, m2_res64 and
 * m2_verdict run the same propagation on a context's state. */
int m2_carry_normalize(uint32_t p, const int64_t* digits, const int64_t* seg_carries, uint32_t seg_digits,
                       uint64_t* out, void* stream);

/* Test hook of the fused column kernel's bounded wait (no GPU fault): raises
 * the epoch flag of column CTA 0 by 2^20, so in the next fused launch CTA 0
 * waits for a flag value that its predecessor never writes; the wait gives up
 * after its limit, the launch completes, and m2_sync reports M2_ETIMEOUT.  The
 * state is then meaningless until m2_set_digits reloads it (which also resets
 * the flags).  M2_EUNSUPPORTED when the context has no fused column pass. */
int m2_test_stall_fused(m2_ctx* ctx);

/* Test hook for stage-by-stage checks of the three-pass path: runs one stage
 * of a squaring on the context's state -- 0: the forward column pass (pending
 * carries, weights, the first log2 R levels of the transform down the columns),
 * 1: the row pass (the remaining forward levels, the centre square, the first
 * inverse levels), 2: the inverse column pass (the last inverse levels,
 * unweight, CRT, carry) -- and copies the transform elements it leaves (h
 * GF(P61^2) pairs of 64-bit words to za_out, h GF(P31^2) pairs of 32-bit words
 * to zb_out; either may be NULL), element r B + c holding row r, column c.
 * Stages 0, 1, 2 in that order make one squaring (stage 2 counts it); between
 * them the digit state is meaningless.  Blocking.  M2_EUNSUPPORTED on the
 * one-CTA path.  The reference's host self-tests compare its fused kernels with
 * its generic chain (mersenne2_gpu.cpp:3200-3240, 3359-3397); this engine's
 * transform uses its own roots and plan, so its stages are checked against an
 * exact model of the arithmetic each stage must perform. */
int m2_test_stage(m2_ctx* ctx, int stage, void* za_out, void* zb_out);

/* ---------------- Gerbicz error check (PRP) ----------------
 * A periodic self-check of a PRP chain (M2_MODE_PRP: x <- x^2 from 3), with
 * rollback to the last verified state.  No reference counterpart: the
 * reference checks nothing between its start and its final residue
 * (mersenne2_gpu.cpp:4778-4882).  With x_k the state after k squarings and k0
 * the last verified iteration, the check product d_t = x_k0 x_(k0+B) ...
 * x_(k0+tB) is updated every B = `block` squarings, and the chain up to
 * k0 + tB is correct, but for a chance of about 1 / M_p, when
 * d_t == x_k0 d_(t-1)^(2^B).  Products a b mod 2^p - 1 are formed as
 * ((a + b)^2 - (a - b)^2) / 4 from two squarings on a second context of the
 * same exponent and transform, which also runs the B verification squarings:
 * every product and square is the engine's own.  Device memory: six vectors
 * of n words plus the second context.  While a check is attached, every
 * squaring of ctx goes through m2_gec_iterate (m2_set_digits on ctx is
 * allowed: a state changed behind the check's back fails the next check). */
typedef struct m2_gec m2_gec;

typedef struct {
    uint32_t verified_iter;  /* k0: iteration of the last verified state */
    uint32_t block;          /* B */
    uint64_t updates;        /* products d <- d x taken */
    uint64_t checks;         /* m2_gec_check calls that verified something */
    uint64_t failures;       /* of those, the ones that found a wrong state */
    double seconds;          /* host wall time spent in updates and checks */
} m2_gec_stats;

/* Starts checking ctx's chain; its current state counts as verified.
 * M2_EUNSUPPORTED for LL and PRP3 contexts, M2_EINVAL for block = 0. */
int m2_gec_create(m2_gec** out, m2_ctx* ctx, uint32_t block);
/* m2_iterate(ctx, k) with the check product updated at every block boundary
 * passed; returns when the last update is done (the squarings after it are
 * still queued on ctx's stream). */
int m2_gec_iterate(m2_gec* g, uint32_t k);
/* Verifies every squaring since the last verified state: the check-product
 * relation up to the last block boundary, and the squarings after it by
 * repeating them on the second context.  M2_OK: the current state is verified
 * and the check restarts from it.  M2_ECHECK: a mismatch; ctx holds the last
 * verified state and iteration again.  *verified_iter (may be NULL) receives
 * the verified iteration either way. */
int m2_gec_check(m2_gec* g, uint32_t* verified_iter);
/* The last verified state (n canonical digits) and its iteration: what a
 * checkpoint file should hold. */
int m2_gec_verified(m2_gec* g, uint64_t* digits, uint32_t* iteration);
int m2_gec_stats_get(m2_gec* g, m2_gec_stats* st);
/* Releases the second context and the host copies; ctx is left as it is. */
void m2_gec_destroy(m2_gec* g);

/* Digit widths (n bytes) of exponent p, without a device; and log2 n. */
int m2_layout(uint32_t p, int* ln, uint64_t* n, uint8_t* widths /* may be NULL */);
/* The same for either field set (M2_FIELDS_*). */
int m2_layout_fields(uint32_t p, int fields, int* ln, uint64_t* n, uint8_t* widths /* may be NULL */);

const char* m2_strerror(int code);

/* Where the most recent CUDA failure of the calling thread happened and the
 * runtime's description of it ("" when none). */
const char* m2_last_error(void);

/* ---------------- batched engine ----------------
 * Runs `count` independent tests to completion (or `iters[i]` squarings when
 * iters != NULL) in persistent launches grouped by transform size, one CTA per
 * test.  res64_out[i] and is_prime_out[i] (may be NULL) receive the results.
 * No reference counterpart: the reference runs one exponent per process
 * (mersenne2_gpu.cpp:3618-4959). */
typedef struct {
    double seconds;          /* device time of the launches */
    uint64_t squarings;      /* total squarings performed */
    uint32_t launches;       /* kernel launches issued */
    uint32_t buckets;        /* distinct transform sizes */
} m2_batch_stats;

int m2_batch_run(const uint32_t* p, const int* modes, const uint32_t* iters, size_t count,
                 uint64_t* res64_out, int* is_prime_out, int device, m2_batch_stats* stats);

/* Threads per transform that m2_batch_run chose for transform size 2^ln on
 * `device` (autotuned on the first batch containing that size: every candidate
 * 32 ... 256 times a sample of the batch's own tests; the carry split follows),
 * and the measured nanoseconds per test-squaring.  M2_EINVAL if not tuned yet. */
int m2_batch_tuned(int device, int ln, int* threads, double* ns_per_test_iter);

/* The full choice of the batch autotuner for transform size 2^ln on `device`
 * (M2_EINVAL if not tuned yet).  The tuner times every valid combination of
 * three knobs on a sample of the batch's own tests:
 *   threads        threads per transform (the reference's -W work-group size,
 *                  mersenne2_gpu.cpp:3668-3672), 32 ... 256;
 *   carry_blocks   segments of the carry, each normalising n / carry_blocks
 *                  digits serially before handing its carry to the next
 *                  (the reference's -B carry block of carry_pairs digit pairs,
 *                  mersenne2_gpu.cpp:3676-3680, 3950-3968): threads, threads/2
 *                  or threads/4 segments;
 *   fused_middle   radix split of the transform's middle: 0 runs the last
 *                  forward level, the centre square and the first inverse level
 *                  as three shared-memory passes (the reference's separate
 *                  forward4 / square_half / backward4 launches,
 *                  mersenne2_gpu.cpp:4512-4531), 1 runs them as one pass over
 *                  pairs of mirror blocks.
 * carry_pairs = n / (2 carry_blocks) is the -B value of that choice. */
typedef struct {
    int threads;
    int carry_blocks;
    int carry_pairs;
    int fused_middle;
    double ns_per_test_iter;  /* measured nanoseconds per test-squaring of the choice */
    double ns_default;        /* the same for the untuned default (h/4 threads, one segment per thread, unfused) */
} m2_batch_tuning_t;
int m2_batch_tuning(int device, int ln, m2_batch_tuning_t* out);

#ifdef __cplusplus
}
#endif
#endif /* M2GPU_H */
