// m2_gec.cu -- Gerbicz error check of a PRP chain (x <- x^2 mod 2^p - 1).
//
// With x_k the state after k squarings and k0 the last verified iteration,
// the check keeps, in device memory, x_k0, the check product D_t, its previous
// value D_(t-1) and the state at the last block boundary.  Products run on a
// second context of the same exponent and transform (mode PRP: plain
// squarings), so the check uses the engine's own kernels:
//   4 a b = (a + b)^2 - (a - b)^2  mod 2^p - 1,
// one sum or difference of canonical digit vectors (k_gec_combine), the
// device carry propagation to canonical digits, a balance, one squaring, and
// the same for the other term.  Without a division by 4 the check product is
// D_t = 4 D_(t-1) x_(k0+tB) = 4^t d_t with d_t = x_k0 x_(k0+B) ... x_(k0+tB),
// and the relation d_t = x_k0 d_(t-1)^(2^B) becomes
//   D_t = Z 4^((t-1)(1 - 2^B)),  Z = 4 x_k0 D_(t-1)^(2^B),
// where Z is formed by the same product and the power of two is a rotation of
// the p-bit residue (2^p == 1), applied on the host once per verification.
// The block products are enqueued without a host wait: the context's stream
// hands the boundary state to the second context's stream through an event,
// and waits for the product through another before its next squaring.
#include "m2_internal.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <new>
#include <vector>

namespace {

using ull = unsigned long long;
using u32 = uint32_t;

__device__ __forceinline__ ull bitpos_at(ull p, int ln, ull j) { return j ? (((p * j) - 1) >> ln) + 1 : 0; }

// out_j = a_j + b_j, or a_j + (2^w_j - 1 - b_j) (a - b mod 2^p - 1, since the
// complement of canonical b is M_p - b): digits below 2^(w_j + 1)
__global__ void k_gec_combine(const ull* __restrict__ a, const ull* __restrict__ b, int subtract,
                              long long* __restrict__ out, ull p, int ln, ull n) {
    for (ull j = blockIdx.x * (ull)blockDim.x + threadIdx.x; j < n; j += (ull)gridDim.x * blockDim.x) {
        const ull w = bitpos_at(p, ln, j + 1) - bitpos_at(p, ln, j);
        const ull m = (1ull << w) - 1;
        out[j] = (long long)(a[j] + (subtract ? m - b[j] : b[j]));
    }
}

__global__ void k_gec_diff(const ull* __restrict__ a, const ull* __restrict__ b, ull n, unsigned* count) {
    unsigned c = 0;
    for (ull j = blockIdx.x * (ull)blockDim.x + threadIdx.x; j < n; j += (ull)gridDim.x * blockDim.x) c += (a[j] != b[j]);
    if (c) atomicAdd(count, c);
}

inline u32 grid_for(ull n) { return (u32)std::min<ull>((n + 255) / 256, 152ull * 8); }

inline ull mask_of(u32 w) { return w >= 64 ? ~0ull : (1ull << w) - 1; }

// v <- v * 2^e mod 2^p - 1 for canonical v (host): bit i of the result is bit
// (i - e) mod p of v
void rotate_up(const m2::Layout& L, std::vector<uint64_t>& v, uint64_t e) {
    const uint64_t p = L.p;
    e %= p;
    if (e == 0) return;
    const uint64_t r = p - e;   // source bit of result bit i: (i + r) mod p
    std::vector<uint64_t> bits(p / 64 + 2, 0);
    for (uint64_t j = 0; j < L.n; ++j) {
        const uint64_t pos = L.bitpos[j], w = L.width[j];
        if (w == 0 || v[j] == 0) continue;
        const uint64_t k = pos >> 6, off = pos & 63;
        bits[k] |= v[j] << off;
        if (off + w > 64) bits[k + 1] |= v[j] >> (64 - off);
    }
    auto get = [&](uint64_t pos, uint64_t len) -> uint64_t {   // len <= 64, pos + len <= p
        if (len == 0) return 0;
        const uint64_t k = pos >> 6, off = pos & 63;
        uint64_t x = bits[k] >> off;
        if (off + len > 64) x |= bits[k + 1] << (64 - off);
        return x & mask_of((u32)len);
    };
    for (uint64_t j = 0; j < L.n; ++j) {
        const uint64_t w = L.width[j], pos = (L.bitpos[j] + r) % p;
        if (pos + w <= p) {
            v[j] = get(pos, w);
        } else {
            const uint64_t lo = p - pos;
            v[j] = get(pos, lo) | (get(0, w - lo) << lo);
        }
    }
}

uint64_t pow2_mod(uint64_t e, uint64_t m) {
    uint64_t r = 1 % m, b = 2 % m;
    for (; e; e >>= 1, b = b * b % m)
        if (e & 1) r = r * b % m;
    return r;
}

double now_s() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

}  // namespace

struct m2_gec {
    m2_ctx* ctx = nullptr;          // the checked chain (owned by the caller)
    m2_ctx* aux = nullptr;          // the check's squarings
    const m2::Layout* L = nullptr;
    u32 block = 0;
    u32 k0 = 0;                     // last verified iteration
    u32 cur = 0;                    // ctx's iteration
    u32 t = 0;                      // products taken since k0
    cudaStream_t cs = nullptr, as = nullptr;     // ctx's and aux's streams
    cudaEvent_t to_aux = nullptr, to_ctx = nullptr;
    // device vectors of n canonical digits
    ull* x0 = nullptr;              // x_k0
    ull* D = nullptr;               // D_t
    ull* Dprev = nullptr;           // D_(t-1)
    ull* xb = nullptr;              // x_(k0+tB)
    ull* sq = nullptr;              // (a + b)^2 inside a product
    ull* tmp = nullptr;
    unsigned* count = nullptr;      // mismatch counter
    m2_gec_stats st{};
};

namespace {

int cuda_rc(cudaError_t e) {
    if (e == cudaSuccess) return M2_OK;
    return e == cudaErrorMemoryAllocation ? M2_ENOMEM : M2_ECUDA;
}

// aux's state <- a +/- b (canonical vectors in device memory), canonical
// digits of the result left in aux's canonical buffer
int combine_into_aux(m2_gec* g, const ull* a, const ull* b, bool subtract, const ull** canon) {
    long long* raw = nullptr;
    int rc = m2i::raw_state(g->aux, &raw);
    if (rc) return rc;
    const m2::Layout& L = *g->L;
    k_gec_combine<<<grid_for(L.n), 256, 0, g->as>>>(a, b, subtract ? 1 : 0, raw, L.p, L.ln, L.n);
    if ((rc = cuda_rc(cudaGetLastError()))) return rc;
    return m2i::canonical(g->aux, canon);
}

// aux's canonical buffer <- v^(2^k) for canonical v in device memory
int square_k(m2_gec* g, const ull* v, u32 k, const ull** canon) {
    ull* buf = nullptr;
    int rc = m2i::canon_buffer(g->aux, &buf);
    if (rc) return rc;
    if (v != buf && (rc = cuda_rc(cudaMemcpyAsync(buf, v, g->L->n * sizeof(ull), cudaMemcpyDeviceToDevice, g->as)))) return rc;
    if ((rc = m2i::load_canon(g->aux, 0))) return rc;
    if ((rc = m2_iterate(g->aux, k))) return rc;
    return m2i::canonical(g->aux, canon);
}

// out = 4 a b mod 2^p - 1: canonical a, b, out in device memory, out distinct
// from a and b; everything on aux's stream
int mul4(m2_gec* g, const ull* a, const ull* b, ull* out) {
    const size_t bytes = g->L->n * sizeof(ull);
    const ull* c = nullptr;
    int rc = combine_into_aux(g, a, b, false, &c);                 // a + b
    if (!rc) rc = square_k(g, c, 1, &c);
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(g->sq, c, bytes, cudaMemcpyDeviceToDevice, g->as));
    if (!rc) rc = combine_into_aux(g, a, b, true, &c);             // a - b
    if (!rc) rc = square_k(g, c, 1, &c);
    if (!rc) rc = combine_into_aux(g, g->sq, c, true, &c);         // (a + b)^2 - (a - b)^2
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(out, c, bytes, cudaMemcpyDeviceToDevice, g->as));
    return rc;
}

// number of digits where two canonical device vectors differ (aux's stream)
int count_diff(m2_gec* g, const ull* a, const ull* b, unsigned* out) {
    int rc = cuda_rc(cudaMemsetAsync(g->count, 0, sizeof(unsigned), g->as));
    if (rc) return rc;
    k_gec_diff<<<grid_for(g->L->n), 256, 0, g->as>>>(a, b, g->L->n, g->count);
    if ((rc = cuda_rc(cudaGetLastError()))) return rc;
    if ((rc = cuda_rc(cudaMemcpyAsync(out, g->count, sizeof(unsigned), cudaMemcpyDeviceToHost, g->as)))) return rc;
    return cuda_rc(cudaStreamSynchronize(g->as));
}

// ctx's current canonical state copied to dst (ctx's stream, then waited for)
int ctx_state(m2_gec* g, ull* dst) {
    const ull* c = nullptr;
    int rc = m2i::canonical(g->ctx, &c);
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(dst, c, g->L->n * sizeof(ull), cudaMemcpyDeviceToDevice, g->cs));
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(g->cs));
    return rc;
}

// the chain restarts from its last verified state: D_0 = x_k0, and x_k0 is
// the last boundary's state
int restart(m2_gec* g) {
    g->t = 0;
    g->cur = g->k0;
    const size_t bytes = g->L->n * sizeof(ull);
    int rc = cuda_rc(cudaMemcpyAsync(g->D, g->x0, bytes, cudaMemcpyDeviceToDevice, g->as));
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(g->xb, g->x0, bytes, cudaMemcpyDeviceToDevice, g->as));
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(g->as));
    return rc;
}

int set_device(const m2_gec* g) { return cuda_rc(cudaSetDevice(m2i::creation_opts(g->ctx).device)); }

void release(m2_gec* g) {
    ull* bufs[] = {g->x0, g->D, g->Dprev, g->xb, g->sq, g->tmp};
    for (ull* b : bufs) if (b) cudaFree(b);
    if (g->count) cudaFree(g->count);
    if (g->to_aux) cudaEventDestroy(g->to_aux);
    if (g->to_ctx) cudaEventDestroy(g->to_ctx);
    m2_destroy(g->aux);
    delete g;
}

}  // namespace

extern "C" {

int m2_gec_create(m2_gec** out, m2_ctx* ctx, uint32_t block) {
    if (!out) return M2_EINVAL;
    *out = nullptr;
    if (!ctx || block == 0) return M2_EINVAL;
    m2_info_t info{};
    int rc = m2_info(ctx, &info);
    if (rc) return rc;
    if (info.mode != M2_MODE_PRP) return M2_EUNSUPPORTED;
    m2_gec* g = new (std::nothrow) m2_gec();
    if (!g) return M2_ENOMEM;
    g->ctx = ctx;
    g->L = &m2i::layout(ctx);
    g->block = block;
    g->cs = m2i::stream(ctx);
    const m2_opts o = m2i::creation_opts(ctx);
    if ((rc = m2_create(&g->aux, info.p, M2_MODE_PRP, &o))) { delete g; return rc; }
    g->as = m2i::stream(g->aux);
    const size_t bytes = g->L->n * sizeof(ull);
    ull** bufs[] = {&g->x0, &g->D, &g->Dprev, &g->xb, &g->sq, &g->tmp};
    rc = set_device(g);
    for (ull** b : bufs)
        if (!rc) rc = cuda_rc(cudaMalloc(b, bytes));
    if (!rc) rc = cuda_rc(cudaMalloc(&g->count, sizeof(unsigned)));
    if (!rc) rc = cuda_rc(cudaEventCreateWithFlags(&g->to_aux, cudaEventDisableTiming));
    if (!rc) rc = cuda_rc(cudaEventCreateWithFlags(&g->to_ctx, cudaEventDisableTiming));
    if (!rc) rc = ctx_state(g, g->x0);
    g->k0 = info.iteration;
    if (!rc) rc = restart(g);
    if (rc) { release(g); return rc; }
    g->st.verified_iter = g->k0;
    g->st.block = block;
    *out = g;
    return M2_OK;
}

int m2_gec_iterate(m2_gec* g, uint32_t k) {
    if (!g) return M2_EINVAL;
    const double t0 = now_s();
    const size_t bytes = g->L->n * sizeof(ull);
    int rc = set_device(g);
    while (k > 0 && !rc) {
        const uint64_t next = (uint64_t)g->k0 + (uint64_t)(g->t + 1) * g->block;
        const u32 step = (u32)std::min<uint64_t>(k, next - g->cur);
        if ((rc = m2_iterate(g->ctx, step))) break;
        g->cur += step;
        k -= step;
        if (g->cur != next) continue;
        // the boundary state to the check's stream, D_(t+1) = 4 D_t x_(k0+(t+1)B),
        // and the chain's next squaring after the product
        const ull* c = nullptr;
        if ((rc = m2i::canonical(g->ctx, &c))) break;
        if ((rc = cuda_rc(cudaMemcpyAsync(g->xb, c, bytes, cudaMemcpyDeviceToDevice, g->cs)))) break;
        if ((rc = cuda_rc(cudaEventRecord(g->to_aux, g->cs)))) break;
        if ((rc = cuda_rc(cudaStreamWaitEvent(g->as, g->to_aux, 0)))) break;
        std::swap(g->D, g->Dprev);
        if ((rc = mul4(g, g->Dprev, g->xb, g->D))) break;
        if ((rc = cuda_rc(cudaEventRecord(g->to_ctx, g->as)))) break;
        if ((rc = cuda_rc(cudaStreamWaitEvent(g->cs, g->to_ctx, 0)))) break;
        ++g->t;
        ++g->st.updates;
    }
    g->st.seconds += now_s() - t0;
    return rc;
}

int m2_gec_check(m2_gec* g, uint32_t* verified_iter) {
    if (!g) return M2_EINVAL;
    const double t0 = now_s();
    const m2::Layout& L = *g->L;
    const size_t bytes = L.n * sizeof(ull);
    const u32 tail = g->cur - (g->k0 + g->t * g->block);
    int rc = set_device(g);
    bool ok = true;
    // the chain and its products done; a kernel that reported an
    // out-of-range carry or a wait that gave up has left a wrong state: the
    // same rollback as a mismatch
    if (!rc) {
        const int s_ctx = m2_sync(g->ctx);
        const int s_aux = cudaStreamSynchronize(g->as) == cudaSuccess ? m2_sync(g->aux) : M2_ECUDA;
        for (const int sv : {s_ctx, s_aux}) {
            if (sv == M2_ESTATE || sv == M2_ETIMEOUT) ok = false;
            else if (sv && !rc) rc = sv;
        }
    }
    if (!rc && ok && (g->t > 0 || tail > 0)) {
        if (g->t > 0) {
            // Z = 4 x_k0 D_(t-1)^(2^B); the chain is right when D_t == Z 4^((t-1)(1 - 2^B))
            const ull* c = nullptr;
            rc = square_k(g, g->Dprev, g->block, &c);
            if (!rc) rc = cuda_rc(cudaMemcpyAsync(g->tmp, c, bytes, cudaMemcpyDeviceToDevice, g->as));
            if (!rc) rc = mul4(g, g->tmp, g->x0, g->Dprev);   // D_(t-1) is not needed afterwards
            std::vector<uint64_t> z, d;
            try {
                z.resize(L.n);
                d.resize(L.n);
            } catch (const std::bad_alloc&) {
                rc = M2_ENOMEM;
            }
            if (!rc) rc = cuda_rc(cudaMemcpyAsync(z.data(), g->Dprev, bytes, cudaMemcpyDeviceToHost, g->as));
            if (!rc) rc = cuda_rc(cudaMemcpyAsync(d.data(), g->D, bytes, cudaMemcpyDeviceToHost, g->as));
            if (!rc) rc = cuda_rc(cudaStreamSynchronize(g->as));
            if (!rc) {
                const uint64_t p = L.p;
                const uint64_t f = (1 + p - pow2_mod(g->block, p)) % p;          // 1 - 2^B mod p
                rotate_up(L, z, 2 * ((uint64_t)(g->t - 1) % p * f % p) % p);     // 4^((t-1)(1 - 2^B))
                ok = (z == d);
            }
        }
        if (!rc && ok) {
            // the current state: the last boundary's, or the squarings after
            // that boundary repeated on the second context
            unsigned diff = 0;
            const ull* ref = g->xb;
            rc = ctx_state(g, g->tmp);
            if (!rc && tail > 0) rc = square_k(g, g->xb, tail, &ref);
            if (!rc) rc = count_diff(g, g->tmp, ref, &diff);
            if (!rc) ok = (diff == 0);
        }
        if (!rc) {
            ++g->st.checks;
            if (ok) {
                g->k0 = g->cur;
                rc = cuda_rc(cudaMemcpyAsync(g->x0, g->tmp, bytes, cudaMemcpyDeviceToDevice, g->as));
            }
        }
    }
    if (!rc && !ok) {
        // back to (x_k0, k0)
        ++g->st.failures;
        ull* buf = nullptr;
        rc = cuda_rc(cudaStreamSynchronize(g->as));
        if (!rc) rc = m2i::canon_buffer(g->ctx, &buf);
        if (!rc) rc = cuda_rc(cudaMemcpyAsync(buf, g->x0, bytes, cudaMemcpyDeviceToDevice, g->cs));
        if (!rc) rc = m2i::load_canon(g->ctx, g->k0);
        if (!rc) rc = m2_sync(g->ctx);
        if (!rc) rc = M2_ECHECK;
    }
    if (!rc || rc == M2_ECHECK) {
        const int r2 = restart(g);
        if (r2) rc = r2;
    }
    g->st.verified_iter = g->k0;
    if (verified_iter) *verified_iter = g->k0;
    g->st.seconds += now_s() - t0;
    return rc;
}

int m2_gec_verified(m2_gec* g, uint64_t* digits, uint32_t* iteration) {
    if (!g) return M2_EINVAL;
    int rc = set_device(g);
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(g->as));
    if (!rc && digits) rc = cuda_rc(cudaMemcpy(digits, g->x0, g->L->n * sizeof(ull), cudaMemcpyDeviceToHost));
    if (!rc && iteration) *iteration = g->k0;
    return rc;
}

int m2_gec_stats_get(m2_gec* g, m2_gec_stats* st) {
    if (!g || !st) return M2_EINVAL;
    *st = g->st;
    return M2_OK;
}

void m2_gec_destroy(m2_gec* g) {
    if (!g) return;
    set_device(g);
    cudaStreamSynchronize(g->as);
    release(g);
}

}  // extern "C"
