// m2_noalloc.cu -- m2_square_noalloc: the three-pass squaring with no device
// allocation at all.
//
// Who needs this: code that may not call cudaMalloc -- a host framework that
// owns all device memory through its own pool and forbids raw allocations,
// latency-critical paths where an allocation can implicitly synchronise the
// device, or callers that run where the allocator is unavailable.  Such a
// caller already holds the digit buffer on the device and only wants the
// residue advanced by k squarings in place.
//
// Everything the three-pass path needs beyond the caller's digits -- the
// dual-field element arrays, the segment carries, the twiddle and weight
// tables and a status word -- lives in one file-scope static __device__ array
// (8 MiB).  Every GPU that loads the library holds it until the process
// exits.  The largest transform that fits is n = 2^18 digits (p <= 9437179);
// the smallest the three-pass plan accepts is n = 128 (p >= 2689).
//
// The array is shared by every call and keeps the last call's contents: each
// call rebuilds the tables and clears the carries it relies on, and two calls
// whose work overlaps on the GPU (different streams, or different threads on
// one device) race on it.  The first call on a device looks the array's device
// address up (cudaGetSymbolAddress, with that device current).
#include "../../include/m2gpu.h"
#include "m2_field.cuh"
#include "m2_host.hpp"
#include "m2_internal.hpp"
#include "m2_kernels.cuh"

#include <cuda_runtime.h>

#include <mutex>

using namespace m2d;

namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;
constexpr unsigned kMaxLogN = 18;
constexpr unsigned kMinLogN = 7;
constexpr int kMaxDevices = 64;

static_assert(kScratchBytes == (size_t(8) << 20), "scratch size is part of the documented contract");

// The scratch.  Host code must never use this symbol as a pointer: its host
// name is a stand-in, not a device address.  Kernels receive the address that
// cudaGetSymbolAddress returned for the current device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }


__device__ __forceinline__ E dpow(E x, unsigned long long e) {
    E r{1, 0, 1, 0};
    while (e) {
        if (e & 1) r = emul(r, x);
        x = esqr(x);
        e >>= 1;
    }
    return r;
}
__device__ __forceinline__ unsigned brev(unsigned i, int bits) { return bits ? (__brev(i) >> (32 - bits)) : 0u; }
// tables hold canonical coordinates (products leave up to P61 + 5)
__device__ __forceinline__ void put_tw(m2k::DTw* t, unsigned i, const E& v) { t[i] = m2k::DTw{fold61(v.a), fold61(v.b), v.c, v.d}; }

// Twiddle and weight tables of this engine, rebuilt on the device:
//   tw4[3(S+j)+a-1] = r^a with r = w_{4S}^{br_S(j)}, tc[j] = w_h^{br_{h/2}(j)},
//   w61/w31[j] = n^-1 (n - p j mod n) mod 61 / 31 (shift 0 for j = 0).
__global__ void k_noalloc_tables(m2k::DTw* tw4, m2k::DTw* tc, unsigned char* w61, unsigned char* w31,
                                 unsigned h, int lh, unsigned p, int ln, E wh, unsigned lr61, unsigned lr31) {
    const unsigned n = 2u * h;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const unsigned r = (unsigned)(((unsigned long long)p * t) & (n - 1));
        w61[t] = t ? (unsigned char)((lr61 * (n - r)) % 61u) : 0;
        w31[t] = t ? (unsigned char)((lr31 * (n - r)) % 31u) : 0;
        if (t < h / 2) put_tw(tc, t, dpow(wh, brev(t, lh - 1)));
        // radix-4 step S owns entries S..2S-1; t in [S, 2S) for exactly one power of two S
        if (t >= 1 && t < h / 2) {
            const int sb = 31 - __clz(t);
            const unsigned S = 1u << sb;
            if ((sb & 1) == 0 && 4u * S <= h) {
                const unsigned j = t - S;
                const E r = dpow(wh, (unsigned long long)(h / (4u * S)) * brev(j, sb));
                const E r2 = esqr(r), r3 = emul(r2, r);
                put_tw(tw4, 3u * t, r); put_tw(tw4, 3u * t + 1, r2); put_tw(tw4, 3u * t + 2, r3);
            }
        }
    }
}

__device__ __forceinline__ unsigned long long bitpos_of(unsigned p, int ln, unsigned long long j) {
    return j ? ((((unsigned long long)p * j) - 1) >> ln) + 1 : 0;
}
__device__ __forceinline__ unsigned width_at(unsigned p, int ln, unsigned long long j) {
    return (unsigned)(bitpos_of(p, ln, j + 1) - bitpos_of(p, ln, j));
}

// Caller digits with |d| < 2^w -> digits within 2^(w-1) + 1 of zero, same
// residue: a digit at or above 2^(w-1) sheds 2^w and hands +1 to the next
// digit, a digit below -2^(w-1) gains 2^w and hands -1 on (the top digit's
// unit goes to digit 0, since 2^p == 1 mod M_p).  Each digit keeps a value in
// [-2^(w-1), 2^(w-1)) and receives at most one unit, so every accepted input
// starts the first squaring inside the headroom the transform size assumes.
__device__ __forceinline__ long long shed(long long x, unsigned w, long long& unit) {
    if (w == 0) { unit = 0; return x; }
    const long long half = 1ll << (w - 1);
    unit = (x >= half) ? 1 : (x < -half ? -1 : 0);
    return x - (unit << w);
}
__global__ void k_noalloc_rebalance(long long* d, const long long* src_copy, unsigned n, unsigned p, int ln) {
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const unsigned jm = (j + n - 1) % n;
        long long unit_out, unit_in;
        const long long out = shed(src_copy[j], width_at(p, ln, j), unit_out);
        shed(src_copy[jm], width_at(p, ln, jm), unit_in);
        d[j] = out + unit_in;
    }
}
__global__ void k_noalloc_copy(long long* dst, const long long* src, unsigned n) {
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) dst[j] = src[j];
}

// Folds the pending segment carries into the digits (the carry step that the
// next squaring would otherwise do first), so the caller gets plain digits.
__global__ void k_noalloc_apply_carries(long long* d, const long long* carries, m2k::LargePlan P) {
    const unsigned long long segs = (unsigned long long)P.R * P.G, seg_digits = 2ull * P.C;
    for (unsigned long long s = blockIdx.x * blockDim.x + threadIdx.x; s < segs; s += gridDim.x * blockDim.x) {
        long long c = carries[(s + segs - 1) % segs];
        const unsigned long long j0 = s * seg_digits;
        for (int u = 0; u <= P.span; ++u) {
            const unsigned long long j = j0 + u;
            if (u < P.span) d[j] = split_balanced64(d[j] + c, width_at(P.p, P.ln, j), c);
            else d[j] += c;
        }
    }
}

int noalloc_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return M2_EUNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr) { cudaGetLastError(); return M2_ECUDA; }
        g_addr[device] = ptr;
    }
    *out = g_addr[device];
    return M2_OK;
}

}  // namespace

extern "C" int m2_square_noalloc(uint32_t p, int mode, int64_t* digits, uint32_t iters, void* stream) {
    if (p < 3 || mode < M2_MODE_LL || mode > M2_MODE_PRP3 || digits == nullptr) return M2_EINVAL;
    const int ln = m2::transform_log2(p);
    if (ln > (int)kMaxLogN || ln < (int)kMinLogN) return M2_EUNSUPPORTED;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) { cudaGetLastError(); return M2_ECUDA; }
    void* base = nullptr;
    int rc = noalloc_address(device, &base);
    if (rc) return rc;

    // exponent layout without host tables: only the scalars are needed here
    m2::Layout L;
    L.p = p; L.ln = ln; L.n = 1ull << ln; L.h = L.n / 2; L.q = p >> ln;
    const int span = m2::carry_span(L);
    // the plan of m2_create's three-pass path; at these sizes (n <= 2^18, rows
    // of at most 512) it runs the generic column and row kernels, never the
    // fused column pass, whose epoch flags and ticket this path does not carry
    m2k::LargePlan P{};
    if (!m2i::plan_large(L, span, 0, P)) return M2_EUNSUPPORTED;
    P.mode = mode;
    const unsigned h = (unsigned)L.h, n = (unsigned)L.n;
    unsigned smax = 0;
    for (unsigned S = 1; 4 * S <= h; S *= 4) smax = S;

    // carve the scratch
    unsigned char* s = static_cast<unsigned char*>(base);
    size_t off = 0;
    auto take = [&](size_t bytes) { unsigned char* q = s + off; off = align256(off + bytes); return q; };
    auto* za = reinterpret_cast<ulonglong2*>(take(16ull * h));
    auto* zb = reinterpret_cast<uint2*>(take(8ull * h));
    auto* car = reinterpret_cast<long long*>(take(8ull * P.R * P.G));
    auto* tw4 = reinterpret_cast<m2k::DTw*>(take(sizeof(m2k::DTw) * 3ull * 2 * (smax ? smax : 1)));
    auto* tc = reinterpret_cast<m2k::DTw*>(take(sizeof(m2k::DTw) * (h / 2)));
    auto* w61 = take(n);
    auto* w31 = take(n);
    auto* status = reinterpret_cast<int*>(take(sizeof(int)));
    if (off > kScratchBytes) return M2_EUNSUPPORTED;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const m2::Dual wh = m2::root_of_unity(h);
    const unsigned lr61 = (unsigned)(((1ull << 60) / n) % 61), lr31 = (unsigned)(((1ull << 30) / n) % 31);
    int lh = 0;
    while ((1u << lh) < h) ++lh;
    const int threads = 256, blocks = (int)((n + threads - 1) / threads);
    k_noalloc_tables<<<blocks, threads, 0, st>>>(tw4, tc, w61, w31, h, lh, p, ln, E{wh.a, wh.b, wh.c, wh.d}, lr61, lr31);
    cudaError_t e = cudaMemsetAsync(car, 0, 8ull * P.R * P.G, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int), st);
    if (e != cudaSuccess) return M2_ECUDA;
    // za is free until the first squaring: it holds the copy the rebalance step reads (8n bytes)
    long long* tmp = reinterpret_cast<long long*>(za);
    k_noalloc_copy<<<blocks, threads, 0, st>>>(tmp, reinterpret_cast<long long*>(digits), n);
    k_noalloc_rebalance<<<blocks, threads, 0, st>>>(reinterpret_cast<long long*>(digits), tmp, n, p, ln);
    if (cudaGetLastError() != cudaSuccess) return M2_ECUDA;

    if (m2k::large_setup(P) != cudaSuccess) return M2_ECUDA;
    // flags and ticket stay null: launch_large_iteration runs the separate
    // column passes only, and launch_large_stage refuses the fused one
    // (cudaErrorInvalidValue) when a plan's buffers carry no flags
    const m2k::LargeBufs bufs{reinterpret_cast<long long*>(digits), car, za, zb, w61, w31, tw4, tc, status};
    for (uint32_t i = 0; i < iters; ++i)
        if (m2k::launch_large_iteration(P, bufs, st) != cudaSuccess) return M2_ECUDA;
    const int cblocks = (int)((P.R * P.G + threads - 1) / threads);
    k_noalloc_apply_carries<<<cblocks, threads, 0, st>>>(reinterpret_cast<long long*>(digits), car, P);
    if (cudaGetLastError() != cudaSuccess) return M2_ECUDA;

    int host_status = 0;
    if (cudaMemcpyAsync(&host_status, status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return M2_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return M2_ECUDA;
    return host_status ? M2_ESTATE : M2_OK;
}
