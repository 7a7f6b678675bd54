// ref_driver.cpp -- runs the reference's OWN kernels (the OpenCL C string KC of
// mersenne2_gpu.cpp, compiled as C++ through ref_shim.hpp) on the host CPU, in
// the order of M2's generic launch plan (mersenne2_gpu.cpp:4327-4765, the
// variants without __local memory), with the reference's own host table code
// (mersenne2_gpu.cpp:75-293, driven as in 3902-3968).
//
// TEST INFRASTRUCTURE ONLY: the parity tests use it to pin oracle/m2_oracle.c
// to the reference itself, and bench.py times it as the reference CPU baseline.
// The reference sources are NOT part of this repository: oracle/build_ref.py
// cuts the two source ranges out of the reference checkout into oracle/_ref/
// (git-ignored) and compiles this file against them.
#include "ref_shim.hpp"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace refshim { thread_local size_t gid = 0; }

// ---- the reference's host math (mersenne2_gpu.cpp:75-293) ----
#include "_ref/ref_host.inc"
// ---- the reference's device kernels (mersenne2_gpu.cpp:295-3026) ----
#include "_ref/ref_kernels.inc"

namespace {

// One kernel launch = every global id of the NDRange, in parallel on the host.
template <class F> void launch(size_t gs, F&& f) {
#pragma omp parallel for schedule(static) if (gs >= 4096)
    for (long i = 0; i < (long)gs; ++i) { refshim::gid = (size_t)i; f(); }
}
template <class F> void launch_serial(F&& f) { refshim::gid = 0; f(); }

struct RefCtx {
    uint32_t p; int mode; uint8_t ln; size_t n, h;
    std::vector<GF> z;                  // device buffer z (M2:4010)
    std::vector<ulong> w;               // packed twiddles, 3 words each (M2:4015)
    std::vector<IW> iw;                 // IBDWT shifts (M2:4016)
    std::vector<uchar> width;           // digit widths (M2:4017)
    std::vector<BlockInfo> blocks;      // carry blocks (M2:3950-3968)
    std::vector<BlockState> states;
    std::vector<CarryWord> carry;
};

}  // namespace

extern "C" {

// carry_pairs: the -B knob (pairs per carry block), clamped to a power of two <= h (M2:3480-3486).
void* ref_create(uint32_t p, int mode /*0 LL, 1 PRP*/, uint32_t carry_pairs) {
    if (p < 3 || (mode != 0 && mode != 1)) return nullptr;
    RefCtx* c = new RefCtx();
    c->p = p; c->mode = mode;
    c->ln = transformsize(p);
    c->n = size_t(1) << c->ln; c->h = c->n / 2;
    const size_t n = c->n, h = c->h;
    // tables, as M2:3902-3944 builds them with its host classes
    std::vector<GF61_31> zh(h), wv(n);
    zh[0] = GF61_31(mode == 0 ? 4u : 3u);
    for (size_t i = 1; i < h; ++i) zh[i] = GF61_31(0u);
    for (size_t s = 1; s <= n / 4; s <<= 1) {
        GF61_31 r = GF61_31::root_nth(2 * s);
        for (size_t j = 0; j < s; ++j) wv[s + j] = r.pow(bitrev(j, s));
    }
    for (size_t s = 1; s <= n / 4; s <<= 1)
        for (size_t j = 0; j < s; ++j) wv[n / 2 + s + j] = wv[s + j].mul(wv[2 * (s + j)]);
    std::vector<uint64_t> wraw(3 * n);
    for (size_t i = 0; i < n; ++i) pack_gf_words(wraw, i, wv[i]);
    c->w.assign(wraw.begin(), wraw.end());
    c->z.resize(h);
    for (size_t i = 0; i < h; ++i) {
        GF g = { zh[i].g61.s0(), zh[i].g61.s1(), zh[i].g31.s0(), zh[i].g31.s1() };
        c->z[i] = g;
    }
    const uint8_t lr61 = GF61::log2_root_two(n), lr31 = GF31::log2_root_two(n);
    c->width.assign(n, 0);
    c->iw.assign(n, IW{0, 0});
    uint32_t o = 0;
    for (size_t j = 0; j <= n; ++j) {
        uint64_t qj = uint64_t(p) * j;
        uint32_t cj = (j == 0) ? 0u : uint32_t(((qj - 1) >> c->ln) + 1u);
        if (j > 0) {
            c->width[j - 1] = uchar(cj - o);
            if (j < n) {
                uint32_t r = uint32_t(qj & (n - 1));
                c->iw[j].w61 = uchar((lr61 * (n - r)) % 61);
                c->iw[j].w31 = uchar((lr31 * (n - r)) % 31);
            }
        }
        o = cj;
    }
    // carry blocks of `carry_pairs` pairs (M2:3950-3968)
    uint32_t cp = std::max<uint32_t>(1u, std::min<uint32_t>(carry_pairs ? carry_pairs : 64u, uint32_t(h)));
    uint32_t pw = 1; while ((pw << 1) <= cp) pw <<= 1;
    for (uint32_t start = 0; start < h;) {
        uint32_t cnt = 0, bits = 0;
        while (start + cnt < h && cnt < pw) { bits += c->width[2 * (start + cnt)] + c->width[2 * (start + cnt) + 1]; ++cnt; }
        c->blocks.push_back(BlockInfo{start, cnt, bits, 0u});
        start += cnt;
    }
    c->states.assign(c->blocks.size(), BlockState{});
    c->carry.assign(c->blocks.size(), CarryWord{0, 0});
    return c;
}

void ref_destroy(void* h) { delete static_cast<RefCtx*>(h); }

int ref_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// threads of the work-item loops from now on (n >= 1): the single-thread row
// of the CPU baseline
void ref_set_threads(int n) {
#ifdef _OPENMP
    if (n >= 1) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// k squarings through M2's generic kernel sequence (M2:4327-4765).
void ref_iterate(void* hp, uint32_t k) {
    RefCtx* c = static_cast<RefCtx*>(hp);
    GF* z = c->z.data(); const ulong* w = c->w.data(); const IW* iw = c->iw.data();
    const uchar* dw = c->width.data();
    const int n = int(c->n), ln = int(c->ln);
    const uint nb = uint(c->blocks.size());
    for (uint32_t it = 0; it < k; ++it) {
        launch(c->h, [&] { weight(z, iw); });
        size_t cur = c->n / 4, s = 1;
        for (; cur > 1; cur /= 4, s *= 4) {
            int si = int(s), mi = int(cur / 2);
            launch(s * size_t(mi), [&] { forward4(z, w, si, mi, n); });
        }
        const int n4 = int(c->h / 2);
        if (cur == 1) {
            launch(size_t(n4), [&] { forward2(z, w, n4); });
            launch(size_t(n4), [&] { square_half(z, w, n); });
            launch(size_t(n4), [&] { backward2(z, w, n4); });
        } else {
            launch(size_t(n4), [&] { square_half(z, w, n); });
        }
        for (size_t bm = (cur == 1) ? 4 : 2, bs = s / 4; bs >= 1; bm *= 4, bs /= 4) {
            int si = int(bs), mi = int(bm / 2);
            launch(bs * size_t(mi), [&] { backward4(z, w, si, mi, n); });
        }
        launch(c->h, [&] { unweight_norm(z, iw, ln); });
        launch(nb, [&] { block_prepare_kernel(z, dw, c->blocks.data(), c->states.data(), nb); });
        launch(nb, [&] { init_block_carry_kernel(c->states.data(), c->carry.data(), nb); });
        if ((nb & 1u) == 0u && nb >= 2u) {
            launch(nb, [&] { block_carry_phase_kernel(z, c->blocks.data(), c->carry.data(), dw, nb, 0u); });
            launch(nb, [&] { block_carry_phase_kernel(z, c->blocks.data(), c->carry.data(), dw, nb, 1u); });
        }
        launch_serial([&] { block_carry_drain_kernel(z, c->blocks.data(), c->carry.data(), dw, nb); });
        if (c->mode == 0) launch_serial([&] { sub_kernel(z, dw, uint(c->h), 2u); });
    }
}

// canonical digits (the all-ones vector == M_p maps to zero, M2:3035-3042)
void ref_get_digits(void* hp, uint64_t* out) {
    RefCtx* c = static_cast<RefCtx*>(hp);
    bool ones = true;
    for (size_t k = 0; k < c->h; ++k) {
        out[2 * k] = c->z[k].s0; out[2 * k + 1] = c->z[k].s1;
        if (out[2 * k] != ((uint64_t(1) << c->width[2 * k]) - 1) || out[2 * k + 1] != ((uint64_t(1) << c->width[2 * k + 1]) - 1)) ones = false;
    }
    if (ones) std::memset(out, 0, sizeof(uint64_t) * c->n);
}

uint64_t ref_n(void* hp) { return static_cast<RefCtx*>(hp)->n; }

}  // extern "C"
