// m2_api.cu -- the C ABI of include/m2gpu.h on top of the kernels.
#include "../../include/m2gpu.h"
#include "m2_host.hpp"
#include "m2_internal.hpp"
#include "m2_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <tuple>
#include <vector>
#include <chrono>
#include <deque>
#include <thread>

using m2::i64;
using m2::u32;
using m2::u64;

namespace {

// ---------------- device twiddle cache (one table set per device and h) ----------------
struct TwTables {
    m2k::DTw* tw4 = nullptr;
    m2k::DTw* tc = nullptr;
    size_t bytes = 0;
};
std::mutex g_tw_mu;
std::map<std::pair<int, u64>, TwTables> g_tw;

cudaMemPool_t ctx_pool(int device);

// Tables of a new transform size come from the stream-ordered pool on a stream
// of their own, so building them waits for nothing else running on the device
// (a cudaMalloc may synchronise the whole device).  Kept until the process ends.
int get_twiddles(int device, u64 h, TwTables& out) {
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto it = g_tw.find({device, h});
    if (it != g_tw.end()) { out = it->second; return M2_OK; }
    m2::Twiddles T = m2::make_twiddles(h);
    TwTables t;
    const size_t b4 = T.tw4.size() * sizeof(m2::Dual), bc = T.tc.size() * sizeof(m2::Dual);
    cudaMemPool_t mp = ctx_pool(device);
    cudaStream_t s = nullptr;
    if (!mp || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); return M2_ECUDA; }
    cudaError_t e = cudaMallocFromPoolAsync((void**)&t.tw4, b4, mp, s);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync((void**)&t.tc, bc, mp, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t.tw4, T.tw4.data(), b4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t.tc, T.tc.data(), bc, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? M2_ENOMEM : M2_ECUDA;
    }
    t.bytes = b4 + bc;
    g_tw[{device, h}] = t;
    out = t;
    return M2_OK;
}

// ---------------- context memory: one stream-ordered pool per device ----------------
// Contexts allocate and free on their own stream (cudaMallocFromPoolAsync /
// cudaFreeAsync), so creating or destroying one never waits for work that other
// contexts have in flight: the serving engine retires tests while others run.
// The pool keeps freed blocks for reuse (release threshold: unlimited).
std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pool;

cudaMemPool_t ctx_pool(int device) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_pool.find(device);
    if (it != g_pool.end()) return it->second;
    cudaMemPoolProps pp{};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = device;
    cudaMemPool_t mp = nullptr;
    if (cudaMemPoolCreate(&mp, &pp) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    uint64_t keep = ~uint64_t(0);
    cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pool[device] = mp;
    return mp;
}

thread_local char g_last_error[256] = "";

// records where a CUDA call failed (readable through m2_last_error) and maps the code
int fail_cuda(const char* where, cudaError_t e) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", where, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? M2_ENOMEM : M2_ECUDA;
}

u32 total_iters_for(u32 p, int mode) {
    if (mode == M2_MODE_LL) return p >= 2 ? p - 2 : 0;
    if (mode == M2_MODE_PRP3) return p - 1;
    return p;
}

// Carry threads of the one-CTA path: a power of two (threads >> shift at most),
// each owning n/Tc >= span+1 digits; 0 selects the single-thread full
// normalization (tiny exponents).
int small_carry_threads(const m2::Layout& L, int span, int threads, int shift = 0) {
    if (L.q < 4) return 0;
    u64 tc = (u64)(threads >> shift);
    if (tc < 1) tc = 1;
    while (tc > 1 && L.n / tc < (u64)span + 1) tc >>= 1;
    if (L.n / tc < (u64)span + 1) return 0;
    return (int)tc;
}

}  // namespace

struct m2_ctx {
    m2::Layout L;
    int mode = M2_MODE_PRP;
    int path = M2_PATH_SMALL;
    u32 iteration = 0;
    int device = 0;
    m2_opts opts{};            // as passed to m2_create, stream cleared
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int span = 0;
    uint64_t bytes = 0;
    // tables
    unsigned char* d_w61 = nullptr;
    unsigned char* d_w31 = nullptr;
    TwTables tw;
    int* d_status = nullptr;
    long long* d_digits = nullptr;
    // small path
    m2k::SmallTest* d_test = nullptr;
    m2k::SmallTest h_test{};   // host copy of the descriptor (the serving engine batches these)
    int threads = 0;
    int carry_threads = 0;
    // large path
    m2k::LargePlan plan{};
    m2k::LargeBufs bufs{};
    long long* d_carries = nullptr;
    ulonglong2* d_za = nullptr;
    uint2* d_zb = nullptr;
    unsigned* d_flags = nullptr;
    uint2* d_aux = nullptr;    // per-element unweighting rotations and digit widths (m2k::LargeBufs::aux)
    bool fused = false;        // inverse and next forward column pass as one cooperative launch
    bool gf61 = false;         // GF(P61^2)-only transform (M2_FIELDS_GF61)
    // GRAPH_ITERS[i] iterations of the three-pass path captured once and replayed
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool graph_failed = false;
    // canonical digits and carry-propagation scratch (allocated on first read)
    unsigned long long* d_canon = nullptr;
    void* d_norm = nullptr;
};

namespace {

template <class T> int dalloc(m2_ctx* c, T** p, size_t bytes) {
    cudaMemPool_t mp = ctx_pool(c->device);
    if (!mp) return M2_ECUDA;
    if (cudaMallocFromPoolAsync((void**)p, bytes, mp, c->stream) != cudaSuccess) { cudaGetLastError(); *p = nullptr; return M2_ENOMEM; }
    c->bytes += bytes;
    return M2_OK;
}

// the fused column kernel's G epoch flags followed by its 64-bit ticket and
// phase counters (G is even, so the counters are 8-byte aligned)
size_t flags_bytes(const m2k::LargePlan& P) { return sizeof(unsigned) * ((size_t)P.G + 4); }


// Iterations of the three-pass path per graph replay, long and short.  With the
// fused column pass a replay of k squarings is 2k + 1 kernels (the forward
// column pass opens it, the inverse one closes it), so the long graph spends
// less on those two passes per squaring.
constexpr uint32_t GRAPH_ITERS[2] = {500, 50};

// Captures GRAPH_ITERS[i] iterations on the context's stream into an executable
// graph (once); replays cost one launch instead of 2 or 3 per iteration.  Not done
// while the caller is capturing the stream itself, or if capture is refused
// (the legacy default stream): launches are then issued one by one.
bool ensure_graph(m2_ctx* c, int i) {
    if (c->graph[i]) return true;
    if (c->graph_failed) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return false;
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        c->graph_failed = true;
        return false;
    }
    cudaError_t e = cudaSuccess;
    e = m2k::launch_large_run(c->plan, c->bufs, GRAPH_ITERS[i], c->fused, c->stream);
    const cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
    if (e == cudaSuccess && ee == cudaSuccess && g && cudaGraphInstantiate(&c->graph[i], g, 0) == cudaSuccess) {
        cudaGraphDestroy(g);
        return true;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    c->graph[i] = nullptr;
    c->graph_failed = true;
    return false;
}

int cuda_err(cudaError_t e) { return e == cudaSuccess ? M2_OK : (e == cudaErrorMemoryAllocation ? M2_ENOMEM : M2_ECUDA); }

int upload_state(m2_ctx* c, const std::vector<u64>& canon) {
    std::vector<i64> bal = m2::balanced_digits(c->L, canon);
    cudaError_t e = cudaMemcpyAsync(c->d_digits, bal.data(), bal.size() * sizeof(i64), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && c->path == M2_PATH_LARGE)
        e = cudaMemsetAsync(c->d_carries, 0, sizeof(i64) * (size_t)c->plan.R * c->plan.G, c->stream);
    if (e == cudaSuccess && c->d_flags) e = cudaMemsetAsync(c->d_flags, 0, flags_bytes(c->plan), c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_err(e);
}

// Full carry propagation of the context's state on its stream (m2_carry.cu):
// canonical digits land in d_canon, the summary flags in the scratch.
int device_canonical(m2_ctx* c, m2k::NormArgs& a) {
    int rc;
    if (!c->d_canon && (rc = dalloc(c, &c->d_canon, c->L.n * sizeof(u64)))) return rc;
    if (!c->d_norm && (rc = dalloc(c, (char**)&c->d_norm, m2k::norm_scratch_bytes(c->L.n)))) return rc;
    a = m2k::NormArgs{};
    a.digits = c->d_digits;
    a.carries = (c->path == M2_PATH_LARGE) ? c->d_carries : nullptr;
    a.seg = (c->path == M2_PATH_LARGE) ? 2ull * c->plan.C : 0;
    a.n = c->L.n; a.p = c->L.p; a.ln = c->L.ln;
    a.out = c->d_canon;
    a.status = c->d_status;
    m2k::norm_bind_scratch(a, c->d_norm);
    const cudaError_t e = m2k::launch_normalize(a, c->stream);
    return e == cudaSuccess ? M2_OK : fail_cuda("carry propagation launch", e);
}

// the first digits (enough for 64 bits) and the summary flags of the canonical state
int read_head(m2_ctx* c, std::vector<u64>& head, unsigned& flags) {
    m2k::NormArgs a;
    int rc = device_canonical(c, a);
    if (rc) return rc;
    head.assign(std::min<u64>(c->L.n, 72), 0);
    cudaError_t e = cudaMemcpyAsync(head.data(), c->d_canon, head.size() * sizeof(u64), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, a.flags, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return fail_cuda("digits read", e);
    return m2_sync(c);
}

}  // namespace

namespace m2i {
// Plan of the three-pass path: rows 4^floor(log2 h / 4), row length h / rows,
// C columns per CTA (carry_pairs when it is a power of two in [4, 16], else 4,
// widened until a segment of 2C digits exceeds the carry span).
bool plan_large(const m2::Layout& L, int span, uint32_t carry_pairs, m2k::LargePlan& P) {
    const int Lh = L.ln - 1;
    if (Lh < 6) return false;
    int L1 = 2 * (Lh / 4);
    if (L1 < 2) L1 = 2;
    const int L2 = Lh - L1;
    P.ln = L.ln; P.L = Lh; P.L1 = L1; P.L2 = L2;
    P.R = 1u << L1; P.B = 1u << L2;
    P.span = span; P.p = L.p;
    // columns per CTA: 4 (the quad-shuffle column kernels' shape for R = 256
    // and 1024, and more CTAs for the small grids of the other mid-size plans)
    uint32_t C = 4;
    if (carry_pairs >= 4 && carry_pairs <= 16 && (carry_pairs & (carry_pairs - 1)) == 0) C = carry_pairs;
    while (2 * C < (uint32_t)span + 1 && C < 16) C <<= 1;
    if (2 * C < (uint32_t)span + 1 || C > P.B) return false;
    P.C = C; P.G = P.B / C;
    // a row pair and a column group must each fit one CTA's shared memory
    // (227 KiB on this GPU): rows of up to 4096 elements, n <= 2^23 digits
    // (p <= 285212671 with both fields, 150994943 with GF(P61^2) alone)
    constexpr uint64_t kSmem = 227ull * 1024;
    if (24ull * 2 * P.B > kSmem || 24ull * P.C * P.R > kSmem) return false;
    return true;
}

const m2::Layout& layout(const m2_ctx* c) { return c->L; }
m2_opts creation_opts(const m2_ctx* c) { return c->opts; }
cudaStream_t stream(const m2_ctx* c) { return c->stream; }

int canonical(m2_ctx* c, const unsigned long long** out) {
    if (cudaSetDevice(c->device) != cudaSuccess) return M2_ECUDA;
    m2k::NormArgs a;
    const int rc = device_canonical(c, a);
    if (!rc) *out = c->d_canon;
    return rc;
}

int raw_state(m2_ctx* c, long long** digits) {
    if (cudaSetDevice(c->device) != cudaSuccess) return M2_ECUDA;
    cudaError_t e = cudaSuccess;
    if (c->path == M2_PATH_LARGE) e = cudaMemsetAsync(c->d_carries, 0, sizeof(i64) * (size_t)c->plan.R * c->plan.G, c->stream);
    if (e != cudaSuccess) return fail_cuda("state reset", e);
    *digits = c->d_digits;
    return M2_OK;
}

int canon_buffer(m2_ctx* c, unsigned long long** buf) {
    int rc;
    if (!c->d_canon && (rc = dalloc(c, &c->d_canon, c->L.n * sizeof(u64)))) return rc;
    if (!c->d_norm && (rc = dalloc(c, (char**)&c->d_norm, m2k::norm_scratch_bytes(c->L.n)))) return rc;
    *buf = c->d_canon;
    return M2_OK;
}

int load_canon(m2_ctx* c, uint32_t iteration) {
    if (cudaSetDevice(c->device) != cudaSuccess) return M2_ECUDA;
    cudaError_t e = m2k::launch_balance(c->d_canon, c->d_digits, c->L.p, c->L.ln, c->L.n, nullptr, c->stream);
    if (e == cudaSuccess && c->path == M2_PATH_LARGE)
        e = cudaMemsetAsync(c->d_carries, 0, sizeof(i64) * (size_t)c->plan.R * c->plan.G, c->stream);
    if (e == cudaSuccess && c->d_flags) e = cudaMemsetAsync(c->d_flags, 0, flags_bytes(c->plan), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream);
    if (e != cudaSuccess) return fail_cuda("state load", e);
    c->iteration = iteration;
    return M2_OK;
}
}  // namespace m2i

extern "C" {

const char* m2_last_error(void) { return g_last_error; }

const char* m2_strerror(int code) {
    switch (code) {
        case M2_OK: return "ok";
        case M2_EINVAL: return "invalid argument";
        case M2_ENOMEM: return "out of device memory";
        case M2_ECUDA: return "CUDA runtime error";
        case M2_ETIMEOUT: return "device wait timed out";
        case M2_ESTATE: return "device reported an out-of-range carry";
        case M2_EUNSUPPORTED: return "unsupported exponent or option";
        case M2_ECHECK: return "error check failed; state reset to the last verified one";
        default: return "unknown error";
    }
}

int m2_layout(uint32_t p, int* ln, uint64_t* n, uint8_t* widths) { return m2_layout_fields(p, M2_FIELDS_DUAL, ln, n, widths); }

int m2_layout_fields(uint32_t p, int fields, int* ln, uint64_t* n, uint8_t* widths) {
    if (p < 3 || (fields != M2_FIELDS_DUAL && fields != M2_FIELDS_GF61)) return M2_EINVAL;
    if (m2::transform_log2(p, fields == M2_FIELDS_GF61 ? 61 : 92) > 30) return M2_EUNSUPPORTED;
    m2::Layout L = m2::make_layout(p, fields == M2_FIELDS_GF61 ? 61 : 92);
    if (ln) *ln = L.ln;
    if (n) *n = L.n;
    if (widths) std::memcpy(widths, L.width.data(), L.n);
    return M2_OK;
}

int m2_create(m2_ctx** out, uint32_t p, int mode, const m2_opts* opts) {
    if (!out) return M2_EINVAL;
    *out = nullptr;
    if (p < 3 || mode < M2_MODE_LL || mode > M2_MODE_PRP3) return M2_EINVAL;
    m2_opts o{};
    if (opts) o = *opts;
    if (o.fields != M2_FIELDS_DUAL && o.fields != M2_FIELDS_GF61) return M2_EINVAL;
    const bool gf61 = (o.fields == M2_FIELDS_GF61);
    if (m2::transform_log2(p, gf61 ? 61 : 92) > 30) return M2_EUNSUPPORTED;
    std::unique_ptr<m2_ctx> c(new (std::nothrow) m2_ctx());
    if (!c) return M2_ENOMEM;
    c->L = m2::make_layout(p, gf61 ? 61 : 92);
    c->gf61 = gf61;
    c->mode = mode;
    c->device = o.device;
    c->opts = o;
    c->opts.stream = nullptr;
    if (cudaSetDevice(o.device) != cudaSuccess) { cudaGetLastError(); return M2_EINVAL; }
    c->span = m2::carry_span(c->L);
    const u64 h = c->L.h;
    int path = o.path;
    // a lone test of h >= 2048 runs faster on the three-pass path's many CTAs
    // than in one CTA (the one-CTA path pays off when many tests share a launch)
    if (path == M2_PATH_AUTO) path = (h <= 1024) ? M2_PATH_SMALL : M2_PATH_LARGE;
    if (path == M2_PATH_SMALL && h > 8192) return M2_EUNSUPPORTED;
    if (path == M2_PATH_LARGE && !m2i::plan_large(c->L, c->span, o.carry_pairs, c->plan)) return M2_EUNSUPPORTED;
    c->path = path;
    if (o.stream) { c->stream = (cudaStream_t)o.stream; }
    else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return M2_ECUDA;
        c->own_stream = true;
    }
    int rc;
    const u64 n = c->L.n;
    if ((rc = get_twiddles(c->device, h, c->tw))) { m2_destroy(c.release()); return rc; }
    m2_ctx* raw = c.get();
    if ((rc = dalloc(raw, &raw->d_w61, n)) || (rc = dalloc(raw, &raw->d_w31, n)) ||
        (rc = dalloc(raw, &raw->d_status, sizeof(int))) || (rc = dalloc(raw, &raw->d_digits, n * sizeof(i64)))) {
        m2_destroy(c.release());
        return rc;
    }
    cudaError_t e = cudaMemcpyAsync(raw->d_w61, raw->L.w61.data(), n, cudaMemcpyHostToDevice, raw->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(raw->d_w31, raw->L.w31.data(), n, cudaMemcpyHostToDevice, raw->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(raw->d_status, 0, sizeof(int), raw->stream);
    if (e != cudaSuccess) { m2_destroy(c.release()); return M2_ECUDA; }
    if (path == M2_PATH_SMALL) {
        raw->threads = m2k::small_threads_for((unsigned)h);
        if (o.wg >= 32 && o.wg <= 256 && (o.wg & (o.wg - 1)) == 0) raw->threads = (int)o.wg;
        raw->carry_threads = small_carry_threads(raw->L, raw->span, raw->threads);
        if (o.carry_pairs > 0 && raw->carry_threads > 0) {
            // -B: segments of about 2 carry_pairs digits, a power of two of them
            int shift = 0;
            while (shift < 8 && (u64)(raw->threads >> (shift + 1)) >= 1 &&
                   2ull * o.carry_pairs * (u64)(raw->threads >> shift) > n)
                ++shift;
            raw->carry_threads = small_carry_threads(raw->L, raw->span, raw->threads, shift);
        }
        if ((rc = dalloc(raw, &raw->d_test, sizeof(m2k::SmallTest)))) { m2_destroy(c.release()); return rc; }
        m2k::SmallTest t{};
        t.digits = raw->d_digits; t.w61 = raw->d_w61; t.w31 = raw->d_w31;
        t.tw4 = raw->tw.tw4; t.tc = raw->tw.tc; t.status = raw->d_status;
        t.p = p; t.iters = 0; t.ln = raw->L.ln; t.mode = mode; t.span = raw->span;
        t.carry_threads = raw->carry_threads;
        t.fuse_middle = o.fused_middle ? 1 : 0;
        t.gf61_only = gf61 ? 1 : 0;
        raw->h_test = t;
        if (cudaMemcpyAsync(raw->d_test, &raw->h_test, sizeof(t), cudaMemcpyHostToDevice, raw->stream) != cudaSuccess) {
            m2_destroy(c.release());
            return M2_ECUDA;
        }
    } else {
        const m2k::LargePlan& P = raw->plan;
        raw->plan.mode = mode;
        raw->plan.gf61 = gf61 ? 1u : 0u;
        if ((rc = dalloc(raw, &raw->d_carries, sizeof(i64) * (size_t)P.R * P.G)) ||
            (rc = dalloc(raw, &raw->d_za, sizeof(ulonglong2) * h)) || (rc = dalloc(raw, &raw->d_zb, sizeof(uint2) * h)) ||
            (rc = dalloc(raw, &raw->d_flags, flags_bytes(P)))) {
            m2_destroy(c.release());
            return rc;
        }
        raw->bufs = m2k::LargeBufs{raw->d_digits, raw->d_carries, raw->d_za, raw->d_zb, raw->d_w61, raw->d_w31,
                                   raw->tw.tw4, raw->tw.tc, raw->d_status, raw->d_flags};
        if (m2k::cols_q_supported(P)) {
            // the inverse column passes' per-element table: the rotation by
            // 2^-(s + ln + 1) that unweights a digit of shift s (mod 61 and mod
            // 31) and the digit widths
            std::vector<uint2> aux(h);
            const uint32_t ln1 = (uint32_t)raw->L.ln + 1;
            auto un = [ln1](uint32_t s, uint32_t m) { const uint32_t t = (s + ln1) % m; return t ? m - t : 0u; };
            for (u64 k = 0; k < h; ++k) {
                const u64 j = 2 * k;
                aux[k].x = un(raw->L.w61[j], 61) | (un(raw->L.w61[j + 1], 61) << 8) | (un(raw->L.w31[j], 31) << 16) |
                           (un(raw->L.w31[j + 1], 31) << 24);
                aux[k].y = (uint32_t)raw->L.width[j] | ((uint32_t)raw->L.width[j + 1] << 8);
            }
            if ((rc = dalloc(raw, &raw->d_aux, sizeof(uint2) * h))) { m2_destroy(c.release()); return rc; }
            if (cudaMemcpyAsync(raw->d_aux, aux.data(), sizeof(uint2) * h, cudaMemcpyHostToDevice, raw->stream) != cudaSuccess ||
                cudaStreamSynchronize(raw->stream) != cudaSuccess) {
                m2_destroy(c.release());
                return M2_ECUDA;
            }
            raw->bufs.aux = raw->d_aux;
        }
        if (m2k::large_setup(P) != cudaSuccess) { m2_destroy(c.release()); return M2_EUNSUPPORTED; }
        raw->fused = m2k::cols_mid_supported(P);
        raw->plan.mid_tickets = (raw->fused && !m2k::cols_mid_cooperative(P)) ? 1u : 0u;
        // the phase barrier measured faster with R = 1024 rows only (n = 2^21)
        raw->plan.mid_barrier = (raw->fused && !P.mid_tickets && P.R == 1024u) ? 1u : 0u;
        raw->bufs.ticket = reinterpret_cast<unsigned long long*>(raw->d_flags + P.G);
        raw->bufs.phase = reinterpret_cast<unsigned long long*>(raw->d_flags + P.G + 2);
    }
    raw->bytes += raw->tw.bytes;
    if ((rc = upload_state(raw, m2::digits_of_small(raw->L, mode == M2_MODE_LL ? 4 : 3)))) { m2_destroy(c.release()); return rc; }
    *out = c.release();
    return M2_OK;
}

int m2_iterate(m2_ctx* c, uint32_t k) {
    if (!c) return M2_EINVAL;
    if (k == 0) return M2_OK;
    if (cudaSetDevice(c->device) != cudaSuccess) return M2_ECUDA;
    cudaError_t e = cudaSuccess;
    if (c->path == M2_PATH_SMALL) {
        e = m2k::launch_small(c->d_test, 1, (unsigned)c->L.h, c->threads, k, c->stream, c->h_test.fuse_middle != 0, c->gf61);
    } else {
        uint32_t left = k;
        for (int i = 0; i < 2; ++i)
            if (left >= GRAPH_ITERS[i] && ensure_graph(c, i))
                for (; left >= GRAPH_ITERS[i] && e == cudaSuccess; left -= GRAPH_ITERS[i]) e = cudaGraphLaunch(c->graph[i], c->stream);
        if (left > 0 && e == cudaSuccess) e = m2k::launch_large_run(c->plan, c->bufs, left, c->fused, c->stream);
    }
    if (e != cudaSuccess) return fail_cuda("m2_iterate launch", e);
    c->iteration += k;
    return M2_OK;
}

int m2_sync(m2_ctx* c) {
    if (!c) return M2_EINVAL;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return M2_ECUDA;
    int st = 0;
    if (cudaMemcpy(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return M2_ECUDA;
    if (st & m2k::ST_WAIT_TIMEOUT) return M2_ETIMEOUT;
    return st ? M2_ESTATE : M2_OK;
}

int m2_get_digits(m2_ctx* c, uint64_t* out) {
    if (!c || !out) return M2_EINVAL;
    m2k::NormArgs a;
    int rc = device_canonical(c, a);
    if (rc) return rc;
    const cudaError_t e = cudaMemcpyAsync(out, c->d_canon, c->L.n * sizeof(u64), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return fail_cuda("digits read", e);
    return m2_sync(c);
}

int m2_set_digits(m2_ctx* c, const uint64_t* digits, uint32_t iteration) {
    if (!c || !digits) return M2_EINVAL;
    if (m2_sync(c) == M2_ECUDA) return M2_ECUDA;
    // canonical input (every digit below 2^width), the usual case: uploaded and
    // balanced on the device, which also checks that it is canonical; anything
    // else is reduced on the host first
    int rc;
    if (!c->d_canon && (rc = dalloc(c, &c->d_canon, c->L.n * sizeof(u64)))) return rc;
    if (!c->d_norm && (rc = dalloc(c, (char**)&c->d_norm, m2k::norm_scratch_bytes(c->L.n)))) return rc;
    unsigned* d_bad = reinterpret_cast<unsigned*>(c->d_norm);   // scratch word, free between reads
    unsigned bad = 0;
    cudaError_t e = cudaMemsetAsync(d_bad, 0, sizeof(unsigned), c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_canon, digits, c->L.n * sizeof(u64), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = m2k::launch_balance(c->d_canon, c->d_digits, c->L.p, c->L.ln, c->L.n, d_bad, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && c->path == M2_PATH_LARGE)
        e = cudaMemsetAsync(c->d_carries, 0, sizeof(i64) * (size_t)c->plan.R * c->plan.G, c->stream);
    if (e == cudaSuccess && c->d_flags) e = cudaMemsetAsync(c->d_flags, 0, flags_bytes(c->plan), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail_cuda("state upload", e);
    if (bad) {
        std::vector<u64> canon;
        try {
            canon = m2::canonical_from_unsigned(c->L, digits);
        } catch (const std::exception&) {
            return M2_EINVAL;
        }
        if ((rc = upload_state(c, canon))) return rc;
        cudaMemset(c->d_status, 0, sizeof(int));
    }
    c->iteration = iteration;
    return M2_OK;
}

int m2_res64(m2_ctx* c, uint64_t* out) {
    if (!c || !out) return M2_EINVAL;
    std::vector<u64> head;
    unsigned flags = 0;
    int rc = read_head(c, head, flags);
    if (rc) return rc;
    u64 r = 0;
    for (u64 j = 0; j < head.size() && c->L.bitpos[j] < 64; ++j) r |= head[j] << c->L.bitpos[j];
    *out = r;
    return M2_OK;
}

int m2_verdict(m2_ctx* c, int* is_prime) {
    if (!c || !is_prime) return M2_EINVAL;
    std::vector<u64> head;
    unsigned flags = 0;
    int rc = read_head(c, head, flags);
    if (rc) return rc;
    u64 want = c->mode == M2_MODE_LL ? 0 : (c->mode == M2_MODE_PRP ? 9 : 3);
    if (c->L.p < 64) want %= (u64(1) << c->L.p) - 1;
    const std::vector<u64> w = m2::digits_of_small(c->L, want);
    // digits from index 8 on are zero when the result was all ones (written as
    // zero) or when no digit there is nonzero
    bool same = (flags & 1u) || !(flags & 2u);
    for (u64 j = 0; j < head.size() && same; ++j) same = (head[j] == w[j]);
    for (u64 j = head.size(); j < w.size() && same; ++j) same = (w[j] == 0);
    *is_prime = same ? 1 : 0;
    return M2_OK;
}

int m2_carry_normalize(uint32_t p, const int64_t* digits, const int64_t* seg_carries, uint32_t seg_digits,
                       uint64_t* out, void* stream) {
    if (p < 3 || !digits || !out) return M2_EINVAL;
    if (m2::transform_log2(p) > 30) return M2_EUNSUPPORTED;
    const int ln = m2::transform_log2(p);
    const u64 n = u64(1) << ln;
    if (seg_carries && (seg_digits == 0 || seg_digits % 8 != 0 || n % seg_digits != 0)) return M2_EINVAL;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return M2_ECUDA;
    cudaMemPool_t mp = ctx_pool(dev);
    if (!mp) return M2_ECUDA;
    cudaStream_t s = (cudaStream_t)stream;
    void* scratch = nullptr;
    const size_t sb = m2k::norm_scratch_bytes(n) + 64;
    cudaError_t e = cudaMallocFromPoolAsync(&scratch, sb, mp, s);
    if (e != cudaSuccess) return fail_cuda("carry scratch", e);
    m2k::NormArgs a{};
    a.digits = reinterpret_cast<const long long*>(digits);
    a.carries = reinterpret_cast<const long long*>(seg_carries);
    a.seg = seg_carries ? seg_digits : 0;
    a.n = n; a.p = p; a.ln = ln;
    a.out = reinterpret_cast<unsigned long long*>(out);
    m2k::norm_bind_scratch(a, scratch);
    a.status = reinterpret_cast<int*>(static_cast<char*>(scratch) + m2k::norm_scratch_bytes(n));
    int st = 0;
    e = cudaMemsetAsync(a.status, 0, sizeof(int), s);
    if (e == cudaSuccess) e = m2k::launch_normalize(a, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, a.status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaFreeAsync(scratch, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail_cuda("carry propagation", e);
    return st ? M2_ESTATE : M2_OK;
}

int m2_test_stall_fused(m2_ctx* c) {
    if (!c) return M2_EINVAL;
    if (!c->fused || !c->d_flags) return M2_EUNSUPPORTED;
    if (cudaSetDevice(c->device) != cudaSuccess) return M2_ECUDA;
    unsigned f0 = 0;
    cudaError_t e = cudaMemcpyAsync(&f0, c->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    f0 += 1u << 20;
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_flags, &f0, sizeof(unsigned), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? M2_OK : fail_cuda("m2_test_stall_fused", e);
}

int m2_test_stage(m2_ctx* c, int stage, void* za_out, void* zb_out) {
    if (!c || stage < 0 || stage > 2) return M2_EINVAL;
    if (c->path != M2_PATH_LARGE) return M2_EUNSUPPORTED;
    if (cudaSetDevice(c->device) != cudaSuccess) return M2_ECUDA;
    cudaError_t e = m2k::launch_large_stage(c->plan, c->bufs, stage, c->stream);
    const size_t h = c->L.h;
    if (e == cudaSuccess && za_out) e = cudaMemcpyAsync(za_out, c->d_za, 16 * h, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && zb_out) e = cudaMemcpyAsync(zb_out, c->d_zb, 8 * h, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail_cuda("m2_test_stage", e);
    if (stage == 2) c->iteration += 1;
    return m2_sync(c);
}

int m2_info(m2_ctx* c, m2_info_t* info) {
    if (!c || !info) return M2_EINVAL;
    std::memset(info, 0, sizeof(*info));
    info->p = c->L.p; info->mode = c->mode; info->ln = c->L.ln; info->n = c->L.n;
    info->iteration = c->iteration;
    info->total_iters = total_iters_for(c->L.p, c->mode);
    info->path = c->path;
    info->span = (uint32_t)c->span;
    if (c->path == M2_PATH_LARGE) { info->rows = c->plan.R; info->row_len = c->plan.B; info->cols_per_cta = c->plan.C; }
    else { info->rows = 1; info->row_len = (uint32_t)c->L.h; info->cols_per_cta = (uint32_t)c->threads; }
    info->device_bytes = c->bytes;
    info->fused_cols = c->fused ? 1u : 0u;
    info->fields = c->gf61 ? M2_FIELDS_GF61 : M2_FIELDS_DUAL;
    return M2_OK;
}

void m2_destroy(m2_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    // stream-ordered frees: they follow the context's queued work and do not
    // wait for other streams; its stream is released once that work is done
    void* bufs[] = {c->d_w61, c->d_w31, c->d_status, c->d_digits, c->d_test, c->d_carries, c->d_za, c->d_zb,
                    c->d_canon, c->d_norm, c->d_flags, c->d_aux};
    if (c->stream)
        for (void* b : bufs) if (b) cudaFreeAsync(b, c->stream);
    for (cudaGraphExec_t g : c->graph)
        if (g) cudaGraphExecDestroy(g);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int m2_profile(m2_ctx* c, uint32_t iters, m2_stage_time* out, int max_stages, int* n_stages) {
    if (!c || !out || max_stages < 1 || iters == 0) return M2_EINVAL;
    if (cudaSetDevice(c->device) != cudaSuccess) return M2_ECUDA;
    // the launch sequence m2_iterate issues for `iters` squarings, one event after each
    std::vector<int> seq;
    if (c->path == M2_PATH_SMALL) seq.push_back(-1);
    else if (c->fused) {
        seq = {0, 1};
        for (uint32_t i = 1; i < iters; ++i) { seq.push_back(m2k::STAGE_MID); seq.push_back(1); }
        seq.push_back(2);
    } else {
        for (uint32_t i = 0; i < iters; ++i) for (int st = 0; st < m2k::LARGE_STAGES; ++st) seq.push_back(st);
    }
    std::vector<cudaEvent_t> ev(seq.size() + 1);
    for (auto& e : ev) if (cudaEventCreate(&e) != cudaSuccess) return M2_ECUDA;
    cudaError_t err = cudaEventRecord(ev[0], c->stream);
    for (size_t i = 0; i < seq.size() && err == cudaSuccess; ++i) {
        if (seq[i] < 0)
            err = m2k::launch_small(c->d_test, 1, (unsigned)c->L.h, c->threads, iters, c->stream, c->h_test.fuse_middle != 0, c->gf61);
        else err = m2k::launch_large_stage(c->plan, c->bufs, seq[i], c->stream);
        if (err == cudaSuccess) err = cudaEventRecord(ev[i + 1], c->stream);
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
    // per stage (in order of first appearance): total time and launches
    std::vector<int> order;
    std::map<int, std::pair<double, uint64_t>> tot;
    if (err == cudaSuccess) {
        for (size_t i = 0; i < seq.size(); ++i) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
            if (!tot.count(seq[i])) order.push_back(seq[i]);
            tot[seq[i]].first += ms;
            tot[seq[i]].second += 1;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return fail_cuda("m2_profile", err);
    c->iteration += iters;
    const int k = std::min((int)order.size(), max_stages);
    for (int i = 0; i < k; ++i) {
        const int st = order[i];
        m2_stage_time& o = out[i];
        std::memset(&o, 0, sizeof(o));
        const char* nm = (st < 0) ? "k_small" : m2k::large_stage_name(st);
        std::strncpy(o.name, nm, sizeof(o.name) - 1);
        o.launches = tot[st].second;
        o.ms_per_launch = tot[st].first / (double)o.launches;
        o.iters_per_launch = (st < 0) ? iters : 1u;
        o.bytes_per_launch = (st < 0) ? 16ull * c->L.n : m2k::large_stage_bytes(c->plan, st);
    }
    if (n_stages) *n_stages = k;
    return M2_OK;
}

uint64_t m2_launches_for(m2_ctx* c, uint32_t k) {
    if (!c || k == 0) return 0;
    if (c->path == M2_PATH_SMALL) return 1ull;
    if (!c->fused) return (uint64_t)m2k::LARGE_STAGES * k;
    // graph replays of GRAPH_ITERS[0] then GRAPH_ITERS[1] squarings, then the
    // rest in one sequence
    uint64_t left = k, n = 0;
    for (int i = 0; i < 2 && !c->graph_failed; ++i) {
        const uint64_t chunks = left / GRAPH_ITERS[i];
        n += chunks * (2ull * GRAPH_ITERS[i] + 1);
        left -= chunks * GRAPH_ITERS[i];
    }
    return n + (left ? 2 * left + 1 : 0);
}

int m2_measure_mul_peak(int device, double* products_per_s) {
    if (!products_per_s) return M2_EINVAL;
    const double r = m2k::measure_wide_mul_rate(device);
    if (r <= 0.0) return M2_ECUDA;
    *products_per_s = r;
    return M2_OK;
}

}  // extern "C"

// ---------------- batched engine ----------------
namespace {

// Launch shape of the one-CTA kernel, tuned per (device, h): every
// combination of threads per transform (32 ... 256), carry segments (threads,
// threads / 2, threads / 4, each segment at least span + 1 digits) and the
// fused or separate transform middle runs a GPU-filling sample of the bucket's
// own tests for TUNE_ITERS squarings on scratch copies of their state; the
// highest rate of test-squarings per second wins.  Cached for the process.
struct Tuned {
    int threads = 0, carry_shift = 0, fuse = 0;
    double ns_per_test_iter = 0.0, ns_default = 0.0;
    int carry_blocks(const m2::Layout& L, int span) const { return small_carry_threads(L, span, threads, carry_shift); }
};
std::mutex g_tune_mu;
std::map<std::pair<int, u64>, Tuned> g_tune;
std::map<std::pair<int, u64>, std::pair<int, int>> g_tune_shape;   // (device, h) -> (carry blocks, n) of the choice
constexpr u32 TUNE_ITERS = 48;

template <class Item>
int tune_bucket(int device, u64 h, const std::vector<Item>& items, const std::vector<m2k::SmallTest>& tests,
                const long long* d_dig, int sms, Tuned& out) {
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find({device, h});
        if (it != g_tune.end()) { out = it->second; return M2_OK; }
    }
    const u64 n = 2 * h;
    const size_t cap = std::min<size_t>(items.size(), (size_t)std::max(sms, 1) * 8);
    long long* scratch = nullptr;
    m2k::SmallTest* d_t = nullptr;
    int* d_st = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (st) cudaStreamDestroy(st);
        cudaFree(scratch); cudaFree(d_t); cudaFree(d_st);
    };
    if (cudaMalloc(&scratch, cap * n * sizeof(i64)) != cudaSuccess || cudaMalloc(&d_t, cap * sizeof(m2k::SmallTest)) != cudaSuccess ||
        cudaMalloc(&d_st, sizeof(int)) != cudaSuccess || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return M2_ENOMEM;
    }
    const int T0 = m2k::small_threads_for((unsigned)h);
    Tuned best;
    best.threads = T0;
    for (int T = 32; T <= 256; T *= 2) {
        for (int shift = 0; shift <= 2; ++shift) {
            // a carry split that the segment length rules out collapses onto a smaller shift: skip repeats
            if (shift > 0 && small_carry_threads(items[0].L, items[0].span, T, shift) ==
                                 small_carry_threads(items[0].L, items[0].span, T, shift - 1))
                continue;
            for (int fuse = 0; fuse <= 1; ++fuse) {
                const int per_sm = m2k::small_ctas_per_sm((unsigned)h, T, fuse != 0);
                const size_t ns = std::min(cap, (size_t)per_sm * (size_t)std::max(sms, 1));
                std::vector<m2k::SmallTest> d(tests.begin(), tests.begin() + ns);
                for (size_t t = 0; t < ns; ++t) {
                    d[t].digits = scratch + t * n;
                    d[t].status = d_st;
                    d[t].carry_threads = small_carry_threads(items[t].L, items[t].span, T, shift);
                    d[t].fuse_middle = fuse;
                }
                cudaError_t e = cudaMemcpyAsync(scratch, d_dig, ns * n * sizeof(i64), cudaMemcpyDeviceToDevice, st);
                if (e == cudaSuccess) e = cudaMemcpyAsync(d_t, d.data(), ns * sizeof(m2k::SmallTest), cudaMemcpyHostToDevice, st);
                if (e == cudaSuccess) e = m2k::launch_small(d_t, (int)ns, (unsigned)h, T, 2, st, fuse != 0);   // warm-up
                if (e == cudaSuccess) e = cudaEventRecord(e0, st);
                if (e == cudaSuccess) e = m2k::launch_small(d_t, (int)ns, (unsigned)h, T, TUNE_ITERS, st, fuse != 0);
                if (e == cudaSuccess) e = cudaEventRecord(e1, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) { cleanup(); return fail_cuda("batch tuning", e); }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                const double ns_per = ms * 1e6 / ((double)ns * TUNE_ITERS);
                if (T == T0 && shift == 0 && fuse == 0) best.ns_default = ns_per;
                if (best.ns_per_test_iter == 0.0 || ns_per < best.ns_per_test_iter) {
                    best.threads = T; best.carry_shift = shift; best.fuse = fuse; best.ns_per_test_iter = ns_per;
                }
            }
        }
    }
    cleanup();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[{device, h}] = best;
    g_tune_shape[{device, h}] = {best.carry_blocks(items[0].L, items[0].span), (int)n};
    out = best;
    return M2_OK;
}

}  // namespace

extern "C" {

int m2_batch_tuned(int device, int ln, int* threads, double* ns_per_test_iter) {
    if (ln < 3 || ln > 14) return M2_EINVAL;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find({device, u64(1) << (ln - 1)});
    if (it == g_tune.end()) return M2_EINVAL;
    if (threads) *threads = it->second.threads;
    if (ns_per_test_iter) *ns_per_test_iter = it->second.ns_per_test_iter;
    return M2_OK;
}

int m2_batch_tuning(int device, int ln, m2_batch_tuning_t* out) {
    if (ln < 3 || ln > 14 || !out) return M2_EINVAL;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const u64 h = u64(1) << (ln - 1);
    auto it = g_tune.find({device, h});
    auto sh = g_tune_shape.find({device, h});
    if (it == g_tune.end() || sh == g_tune_shape.end()) return M2_EINVAL;
    out->threads = it->second.threads;
    out->carry_blocks = sh->second.first;
    out->carry_pairs = sh->second.first ? sh->second.second / (2 * sh->second.first) : 0;
    out->fused_middle = it->second.fuse;
    out->ns_per_test_iter = it->second.ns_per_test_iter;
    out->ns_default = it->second.ns_default;
    return M2_OK;
}

// Tests are bucketed by transform length h; every bucket is one persistent
// launch (CTAs pull test indices from a device counter, longest tests first)
// with its tuned threads per transform, all buckets run concurrently on their
// own streams, and the whole set of launches is captured into one CUDA graph.
int m2_batch_run(const uint32_t* p, const int* modes, const uint32_t* iters, size_t count,
                 uint64_t* res64_out, int* is_prime_out, int device, m2_batch_stats* stats) {
    if (!p || count == 0) return M2_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return M2_EINVAL; }
    struct Item { size_t idx; m2::Layout L; int mode; u32 iters; int span; };
    std::map<u64, std::vector<Item>> buckets;
    for (size_t i = 0; i < count; ++i) {
        const int mode = modes ? modes[i] : M2_MODE_PRP;
        if (p[i] < 3 || mode < M2_MODE_LL || mode > M2_MODE_PRP3) return M2_EINVAL;
        if (m2::transform_log2(p[i]) > 14) return M2_EUNSUPPORTED;   // h <= 8192
        Item it;
        it.idx = i; it.L = m2::make_layout(p[i]); it.mode = mode;
        it.iters = iters ? iters[i] : total_iters_for(p[i], mode);
        it.span = m2::carry_span(it.L);
        buckets[it.L.h].push_back(std::move(it));
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    struct Dev {
        std::vector<void*> allocs;
        std::vector<cudaStream_t> streams;
        std::vector<cudaEvent_t> events;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        ~Dev() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            for (auto e : events) cudaEventDestroy(e);
            for (auto s : streams) cudaStreamDestroy(s);
            for (auto a : allocs) cudaFree(a);
        }
    } dv;
    auto dmal = [&](void** ptr, size_t bytes) -> int {
        if (cudaMalloc(ptr, bytes) != cudaSuccess) { cudaGetLastError(); return M2_ENOMEM; }
        dv.allocs.push_back(*ptr);
        return M2_OK;
    };
    struct Launch { u64 h; int threads; int ntests; int grid; m2k::SmallTest* d_tests; int* d_queue; long long* d_dig; std::vector<Item>* items; bool fuse; };
    std::vector<Launch> launches;
    uint64_t squarings = 0;
    for (auto& kv : buckets) {
        const u64 h = kv.first;
        std::vector<Item>& items = kv.second;
        std::sort(items.begin(), items.end(), [](const Item& a, const Item& b) { return a.iters > b.iters; });
        const u64 n = 2 * h;
        const size_t nt = items.size();
        TwTables tw;
        int rc = get_twiddles(device, h, tw);
        if (rc) return rc;
        long long* d_dig = nullptr; unsigned char* d_w = nullptr; m2k::SmallTest* d_tests = nullptr; int* d_q = nullptr;
        if ((rc = dmal((void**)&d_dig, nt * n * sizeof(i64))) || (rc = dmal((void**)&d_w, nt * n * 2)) ||
            (rc = dmal((void**)&d_tests, nt * sizeof(m2k::SmallTest))) || (rc = dmal((void**)&d_q, 2 * sizeof(int))))
            return rc;
        int threads = m2k::small_threads_for((unsigned)h);
        std::vector<i64> dig(nt * n);
        std::vector<unsigned char> w(nt * n * 2);
        std::vector<m2k::SmallTest> tests(nt);
        for (size_t t = 0; t < nt; ++t) {
            const Item& it = items[t];
            std::vector<i64> b = m2::balanced_digits(it.L, m2::digits_of_small(it.L, it.mode == M2_MODE_LL ? 4 : 3));
            std::copy(b.begin(), b.end(), dig.begin() + t * n);
            std::copy(it.L.w61.begin(), it.L.w61.end(), w.begin() + t * 2 * n);
            std::copy(it.L.w31.begin(), it.L.w31.end(), w.begin() + t * 2 * n + n);
            m2k::SmallTest& T = tests[t];
            T.digits = d_dig + t * n; T.w61 = d_w + t * 2 * n; T.w31 = d_w + t * 2 * n + n;
            T.tw4 = tw.tw4; T.tc = tw.tc; T.status = d_q + 1;
            T.p = it.L.p; T.iters = it.iters; T.ln = it.L.ln; T.mode = it.mode; T.span = it.span;
            T.carry_threads = small_carry_threads(it.L, it.span, threads);
            squarings += it.iters;
        }
        if (cudaMemcpy(d_dig, dig.data(), dig.size() * sizeof(i64), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(d_w, w.data(), w.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return M2_ECUDA;
        Tuned tn;
        if ((rc = tune_bucket(device, h, items, tests, d_dig, sms, tn))) return rc;
        threads = tn.threads;
        for (size_t t = 0; t < nt; ++t) {
            tests[t].carry_threads = small_carry_threads(items[t].L, items[t].span, threads, tn.carry_shift);
            tests[t].fuse_middle = tn.fuse;
        }
        if (cudaMemcpy(d_tests, tests.data(), tests.size() * sizeof(m2k::SmallTest), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemset(d_q, 0, 2 * sizeof(int)) != cudaSuccess)
            return M2_ECUDA;
        const int per_sm = m2k::small_ctas_per_sm((unsigned)h, threads, tn.fuse != 0);
        const int grid = (int)std::min<size_t>(nt, (size_t)per_sm * (size_t)std::max(sms, 1));
        launches.push_back(Launch{h, threads, (int)nt, grid, d_tests, d_q, d_dig, &items, tn.fuse != 0});
    }
    // capture: fork from stream 0 to one stream per bucket, join back
    dv.streams.resize(launches.size() + 1);
    for (auto& s : dv.streams) if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return M2_ECUDA;
    dv.events.resize(launches.size() + 3);
    for (auto& e : dv.events) if (cudaEventCreate(&e) != cudaSuccess) return M2_ECUDA;
    cudaStream_t s0 = dv.streams[0];
    if (cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return M2_ECUDA;
    cudaEventRecord(dv.events[0], s0);
    for (size_t b = 0; b < launches.size(); ++b) {
        cudaStream_t sb = dv.streams[b + 1];
        cudaStreamWaitEvent(sb, dv.events[0], 0);
        const Launch& l = launches[b];
        m2k::launch_small_persistent(l.d_tests, l.ntests, (unsigned)l.h, l.threads, l.d_queue, l.grid, sb, l.fuse);
        cudaEventRecord(dv.events[b + 3], sb);
        cudaStreamWaitEvent(s0, dv.events[b + 3], 0);
    }
    if (cudaStreamEndCapture(s0, &dv.graph) != cudaSuccess) return M2_ECUDA;
    if (cudaGraphInstantiate(&dv.exec, dv.graph, 0) != cudaSuccess) return M2_ECUDA;
    cudaEvent_t t0 = dv.events[1], t1 = dv.events[2];
    cudaEventRecord(t0, s0);
    if (cudaGraphLaunch(dv.exec, s0) != cudaSuccess) return M2_ECUDA;
    cudaEventRecord(t1, s0);
    if (cudaStreamSynchronize(s0) != cudaSuccess) return M2_ECUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    int status_any = 0;
    for (const Launch& l : launches) {
        int st = 0;
        if (cudaMemcpy(&st, l.d_queue + 1, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return M2_ECUDA;
        status_any |= st;
        const u64 n = 2 * l.h;
        std::vector<i64> dig((size_t)l.ntests * n);
        if (cudaMemcpy(dig.data(), l.d_dig, dig.size() * sizeof(i64), cudaMemcpyDeviceToHost) != cudaSuccess) return M2_ECUDA;
        for (int t = 0; t < l.ntests; ++t) {
            const Item& it = (*l.items)[t];
            std::vector<i64> d(dig.begin() + (size_t)t * n, dig.begin() + (size_t)(t + 1) * n);
            std::vector<u64> canon;
            try { canon = m2::canonical_digits(it.L, d, {}, 0); } catch (const std::exception&) { return M2_ESTATE; }
            if (res64_out) res64_out[it.idx] = m2::res64_of(it.L, canon);
            if (is_prime_out) {
                const u64 want = it.mode == M2_MODE_LL ? 0 : (it.mode == M2_MODE_PRP ? 9 : 3);
                is_prime_out[it.idx] = m2::equals_small(it.L, canon, want) ? 1 : 0;
            }
        }
    }
    if (stats) {
        stats->seconds = ms * 1e-3;
        stats->squarings = squarings;
        stats->launches = (uint32_t)launches.size();
        stats->buckets = (uint32_t)buckets.size();
    }
    return status_any ? M2_ESTATE : M2_OK;
}

}  // extern "C"

// ---------------- serving engine ----------------
// Lanes run independently: the one-CTA tests of one transform size form one
// lane (one launch advances all of them), every three-pass test is a lane of
// its own (its context's stream).  A step starts the next quantum on every idle
// lane, then waits (bounded) until at least one lane has finished and accounts
// for it, so a long quantum of a large test never holds back small ones.
namespace {

struct SrvItem {
    uint64_t id = 0;
    uint32_t p = 0;
    int mode = 0;
    uint32_t total = 0, done = 0;
    uint32_t inflight = 0;       // squarings launched and not yet accounted
    m2_ctx* ctx = nullptr;
    cudaEvent_t ev = nullptr;    // three-pass tests: end of the quantum in flight
    uint64_t bytes = 0;
    double t_submit = 0, t_admit = 0;
};

struct SrvBucket {
    m2k::SmallTest* d_tests = nullptr;
    m2k::SmallTest* h_tests = nullptr;   // pinned staging of the descriptors
    int* d_status = nullptr;             // status word of each member for this launch
    int* h_status = nullptr;             // pinned copy, read once the launch is done
    size_t cap = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    std::vector<uint64_t> members;       // keys of the tests in the launch in flight
    std::vector<uint32_t> ks;
    bool busy = false;
};

// device memory a test will hold (digits, weights, status, descriptor; the
// element arrays and carries of the three-pass path); twiddles are shared
uint64_t srv_estimate(uint32_t p) {
    const int ln = m2::transform_log2(p);
    const uint64_t n = uint64_t(1) << ln, h = n / 2;
    uint64_t b = 10 * n + 512;
    if (h > 8192) b += 24 * h + 8 * (h / 4) + 4096;
    return b;
}

// longest a step waits for a lane to finish before reporting M2_ETIMEOUT
constexpr double SRV_WAIT_LIMIT_S = 600.0;

}  // namespace

struct m2_server {
    int device = 0;
    uint64_t budget = 0;
    uint32_t quantum = 1000;
    std::deque<SrvItem> queue;
    std::map<uint64_t, SrvItem> active;   // key: admission order
    uint64_t next_key = 0;
    std::deque<m2_srv_result> finished;
    std::map<u64, SrvBucket> buckets;
    uint64_t resident = 0, squarings = 0, completed = 0;
    uint32_t steps = 0, launches = 0;
    std::chrono::steady_clock::time_point t0;
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

void srv_retire(m2_server* s, SrvItem& it, int status) {
    m2_srv_result r{};
    r.id = it.id; r.p = it.p; r.mode = it.mode; r.iters = it.done; r.status = status;
    r.t_submit = it.t_submit; r.t_admit = it.t_admit;
    if (it.ctx) {
        r.n = it.ctx->L.n;
        if (status == M2_OK) {
            int rc = m2_res64(it.ctx, &r.res64);
            if (rc == M2_OK) rc = m2_verdict(it.ctx, &r.is_prime);
            r.status = rc;
        }
        m2_destroy(it.ctx);
        it.ctx = nullptr;
    }
    if (it.ev) { cudaEventDestroy(it.ev); it.ev = nullptr; }
    r.t_done = s->now();
    s->resident -= it.bytes;
    s->completed++;
    s->finished.push_back(r);
}

int srv_bucket_reserve(SrvBucket& b, size_t need) {
    cudaError_t e;
    if (!b.stream && (e = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail_cuda("server stream", e);
    if (!b.ev && (e = cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming)) != cudaSuccess)
        return fail_cuda("server event", e);
    if (b.cap >= need) return M2_OK;
    cudaFree(b.d_tests); cudaFree(b.d_status); cudaFreeHost(b.h_tests); cudaFreeHost(b.h_status);
    b.d_tests = nullptr; b.d_status = nullptr; b.h_tests = nullptr; b.h_status = nullptr;
    const size_t cap = std::max<size_t>({need, 2 * b.cap, 64});
    if ((e = cudaMalloc(&b.d_tests, cap * sizeof(m2k::SmallTest))) != cudaSuccess ||
        (e = cudaMalloc(&b.d_status, cap * sizeof(int))) != cudaSuccess ||
        (e = cudaMallocHost(&b.h_tests, cap * sizeof(m2k::SmallTest))) != cudaSuccess ||
        (e = cudaMallocHost(&b.h_status, cap * sizeof(int))) != cudaSuccess) {
        b.cap = 0;
        return fail_cuda("server descriptors", e);
    }
    b.cap = cap;
    return M2_OK;
}

// starts a quantum on every idle lane
int srv_launch(m2_server* s) {
    std::map<u64, std::vector<uint64_t>> small;
    for (auto& kv : s->active) {
        SrvItem& it = kv.second;
        if (it.inflight) continue;
        if (it.ctx->path == M2_PATH_SMALL) {
            auto b = s->buckets.find(it.ctx->L.h);
            if (b == s->buckets.end() || !b->second.busy) small[it.ctx->L.h].push_back(kv.first);
            continue;
        }
        const uint32_t k = std::min(s->quantum, it.total - it.done);
        int rc = m2_iterate(it.ctx, k);
        if (rc) return rc;
        cudaError_t e = cudaEventRecord(it.ev, it.ctx->stream);
        if (e != cudaSuccess) return fail_cuda("server event record", e);
        it.inflight = k;
        s->launches += (uint32_t)m2_launches_for(it.ctx, k);
    }
    for (auto& kv : small) {
        SrvBucket& b = s->buckets[kv.first];
        const size_t cnt = kv.second.size();
        int rc = srv_bucket_reserve(b, cnt);
        if (rc) return rc;
        b.members = kv.second;
        b.ks.resize(cnt);
        // one launch per transform size: the batch autotuner's shape for it when
        // cached, else the first member's; every member gets the launch's variant
        const m2_ctx* c0 = s->active[kv.second[0]].ctx;
        Tuned tn;
        bool tuned = false;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto f = g_tune.find({s->device, kv.first});
            if (f != g_tune.end()) { tn = f->second; tuned = true; }
        }
        const int threads = tuned ? tn.threads : c0->threads;
        const bool fuse = tuned ? tn.fuse != 0 : c0->h_test.fuse_middle != 0;
        for (size_t j = 0; j < cnt; ++j) {
            SrvItem& it = s->active[kv.second[j]];
            b.ks[j] = std::min(s->quantum, it.total - it.done);
            m2k::SmallTest t = it.ctx->h_test;
            t.iters = b.ks[j];
            t.fuse_middle = fuse ? 1 : 0;
            if (tuned) t.carry_threads = small_carry_threads(it.ctx->L, it.ctx->span, threads, tn.carry_shift);
            t.status = b.d_status + j;
            b.h_tests[j] = t;
        }
        cudaError_t e = cudaMemsetAsync(b.d_status, 0, cnt * sizeof(int), b.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(b.d_tests, b.h_tests, cnt * sizeof(m2k::SmallTest), cudaMemcpyHostToDevice, b.stream);
        if (e != cudaSuccess) return fail_cuda("server descriptor upload", e);
        if ((e = m2k::launch_small(b.d_tests, (int)cnt, (unsigned)kv.first, threads, 0u, b.stream, fuse)) != cudaSuccess)
            return fail_cuda("server small-test launch", e);
        e = cudaMemcpyAsync(b.h_status, b.d_status, cnt * sizeof(int), cudaMemcpyDeviceToHost, b.stream);
        if (e == cudaSuccess) e = cudaEventRecord(b.ev, b.stream);
        if (e != cudaSuccess) return fail_cuda("server status readback", e);
        for (size_t j = 0; j < cnt; ++j) s->active[kv.second[j]].inflight = b.ks[j];
        b.busy = true;
        s->launches++;
    }
    return M2_OK;
}

// accounts for every lane whose quantum has finished; *lanes = how many
int srv_harvest(m2_server* s, int* lanes, bool* busy_left) {
    *lanes = 0;
    *busy_left = false;
    for (auto& kv : s->buckets) {
        SrvBucket& b = kv.second;
        if (!b.busy) continue;
        const cudaError_t e = cudaEventQuery(b.ev);
        if (e == cudaErrorNotReady) { *busy_left = true; continue; }
        if (e != cudaSuccess) return fail_cuda("server small-test wait", e);
        b.busy = false;
        ++*lanes;
        for (size_t j = 0; j < b.members.size(); ++j) {
            auto f = s->active.find(b.members[j]);
            SrvItem& it = f->second;
            const uint32_t k = b.ks[j];
            it.inflight = 0;
            it.done += k;
            it.ctx->iteration += k;
            s->squarings += k;
            const int st = b.h_status[j] ? M2_ESTATE : M2_OK;
            if (st != M2_OK || it.done >= it.total) { srv_retire(s, it, st); s->active.erase(f); }
        }
        b.members.clear();
    }
    for (auto f = s->active.begin(); f != s->active.end();) {
        SrvItem& it = f->second;
        if (it.ctx->path != M2_PATH_LARGE || !it.inflight) { ++f; continue; }
        const cudaError_t e = cudaEventQuery(it.ev);
        if (e == cudaErrorNotReady) { *busy_left = true; ++f; continue; }
        if (e != cudaSuccess) return fail_cuda("server large-test wait", e);
        ++*lanes;
        it.done += it.inflight;
        s->squarings += it.inflight;
        it.inflight = 0;
        const int st = m2_sync(it.ctx);
        if (st != M2_OK || it.done >= it.total) { srv_retire(s, it, st); f = s->active.erase(f); }
        else ++f;
    }
    return M2_OK;
}

}  // namespace

extern "C" {

int m2_srv_create(m2_server** out, int device, uint64_t budget_bytes, uint32_t quantum) {
    if (!out || budget_bytes == 0) return M2_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return M2_EINVAL; }
    m2_server* s = new (std::nothrow) m2_server();
    if (!s) return M2_ENOMEM;
    s->device = device;
    s->budget = budget_bytes;
    s->quantum = quantum ? quantum : 1000;
    s->t0 = std::chrono::steady_clock::now();
    *out = s;
    return M2_OK;
}

int m2_srv_submit(m2_server* s, uint64_t id, uint32_t p, int mode, uint32_t iters) {
    if (!s || p < 3 || mode < M2_MODE_LL || mode > M2_MODE_PRP3) return M2_EINVAL;
    if (m2::transform_log2(p) > 30) return M2_EUNSUPPORTED;
    SrvItem it;
    it.id = id; it.p = p; it.mode = mode;
    const uint32_t full = total_iters_for(p, mode);
    it.total = iters ? std::min(iters, full) : full;
    it.bytes = srv_estimate(p);
    if (it.bytes > s->budget) return M2_ENOMEM;   // could never be admitted: refused, not queued
    it.t_submit = s->now();
    s->queue.push_back(it);
    return M2_OK;
}

int m2_srv_step(m2_server* s) {
    if (!s) return M2_EINVAL;
    if (cudaSetDevice(s->device) != cudaSuccess) return M2_ECUDA;
    // admission: FIFO while the next test fits the budget
    while (!s->queue.empty() && s->resident + s->queue.front().bytes <= s->budget) {
        SrvItem it = s->queue.front();
        s->queue.pop_front();
        m2_opts o{};
        o.device = s->device;
        // up to h = 8192 a test joins its size's shared one-CTA launch
        o.path = (m2::transform_log2(it.p) <= 14) ? M2_PATH_SMALL : M2_PATH_LARGE;
        const int rc = m2_create(&it.ctx, it.p, it.mode, &o);
        it.t_admit = s->now();
        s->resident += it.bytes;
        if (rc != M2_OK) { it.ctx = nullptr; srv_retire(s, it, rc); continue; }
        // from now on the test holds what its context allocated (shared tables excluded)
        const uint64_t own = it.ctx->bytes - it.ctx->tw.bytes;
        s->resident = s->resident - it.bytes + own;
        it.bytes = own;
        if (it.total == 0) { srv_retire(s, it, M2_OK); continue; }
        if (it.ctx->path == M2_PATH_LARGE) {
            const cudaError_t e = cudaEventCreateWithFlags(&it.ev, cudaEventDisableTiming);
            if (e != cudaSuccess) { srv_retire(s, it, fail_cuda("server event", e)); continue; }
        }
        s->active.emplace(s->next_key++, it);
    }
    if (s->active.empty()) return M2_OK;
    s->steps++;
    int rc = srv_launch(s);
    if (rc) return rc;
    // wait until a lane finishes (polling; bounded)
    const auto t_start = std::chrono::steady_clock::now();
    for (;;) {
        int lanes = 0;
        bool busy = false;
        if ((rc = srv_harvest(s, &lanes, &busy))) return rc;
        if (lanes > 0 || !busy) return M2_OK;
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() > SRV_WAIT_LIMIT_S) {
            std::snprintf(g_last_error, sizeof(g_last_error), "m2_srv_step: no lane finished within %.0f s", SRV_WAIT_LIMIT_S);
            return M2_ETIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int m2_srv_poll(m2_server* s, m2_srv_result* out, int max, int* n_out) {
    if (!s || (!out && max > 0)) return M2_EINVAL;
    int n = 0;
    while (n < max && !s->finished.empty()) { out[n++] = s->finished.front(); s->finished.pop_front(); }
    if (n_out) *n_out = n;
    return M2_OK;
}

int m2_srv_stats_get(m2_server* s, m2_srv_stats* st) {
    if (!s || !st) return M2_EINVAL;
    st->queued = (uint32_t)s->queue.size();
    st->active = (uint32_t)s->active.size();
    st->resident_bytes = s->resident;
    st->budget_bytes = s->budget;
    st->squarings = s->squarings;
    st->completed = s->completed;
    st->steps = s->steps;
    st->launches = s->launches;
    return M2_OK;
}

int m2_srv_active_get(m2_server* s, m2_srv_progress* out, int max, int* n_out) {
    if (!s || (!out && max > 0)) return M2_EINVAL;
    int n = 0;
    for (const auto& kv : s->active) {
        if (n >= max) break;
        const SrvItem& it = kv.second;
        m2_srv_progress& g = out[n++];
        g.id = it.id; g.p = it.p; g.done = it.done; g.total = it.total; g.inflight = it.inflight;
        g.n = it.ctx ? it.ctx->L.n : 0;
        g.device_bytes = it.bytes;
        g.t_submit = it.t_submit; g.t_admit = it.t_admit;
    }
    if (n_out) *n_out = n;
    return M2_OK;
}

void m2_srv_destroy(m2_server* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    for (auto& kv : s->buckets)
        if (kv.second.stream) cudaStreamSynchronize(kv.second.stream);
    for (auto& kv : s->active) {
        if (kv.second.ctx) { m2_sync(kv.second.ctx); m2_destroy(kv.second.ctx); }
        if (kv.second.ev) cudaEventDestroy(kv.second.ev);
    }
    for (auto& kv : s->buckets) {
        SrvBucket& b = kv.second;
        cudaFree(b.d_tests); cudaFree(b.d_status); cudaFreeHost(b.h_tests); cudaFreeHost(b.h_status);
        if (b.ev) cudaEventDestroy(b.ev);
        if (b.stream) cudaStreamDestroy(b.stream);
    }
    delete s;
}

}  // extern "C"
