// mixed_engine.cuh -- device side of the mixed-precision engine, shared by
// mixed.cu (host side, launches) and the mixed_k*.cu units, each of which
// defines MSG_MIXED_KERNEL_BODY and explicitly instantiates one (kind,
// d = 3 only) variant of k_engine_mixed, so that the six variants compile in
// parallel.
#pragma once
// The mixed-precision engine: the LU trailing updates run on the
// tcgen05 tensor cores as exact products of bf16 slices, everything else in
// double-float (FP32 hi + lo) on the FP32 pipe: the panel, the TRSM, the
// epilogue and, for d = 3, the whole matrix assembly; the pivot reciprocals,
// ln and the d = 2 Green functions (K_nu) in FP64.
//
// Trailing update C -= A B (A: m x K panel, B: K x nn rows, K <= 32, complex):
//  * every row of A (column of B) is scaled by a power of two so its largest
//    |Re|, |Im| lies in [1/2, 1), then cut into NS integer slices
//    x 2^(8-e) = s0 + s1 2^-9 + ... + s_{NS-1} 2^-9(NS-1) (|s_k| <= 256);
//    slice k is stored as the bf16 value s_k 2^-9k, which is exact (NS = 4:
//    35 bits; NS = 6: 53 bits, the whole double-float);
//  * the slice pairs (i, j) with i + j < NS are multiplied; level l = i + j is
//    accumulated in its own TMEM accumulator for l < NG - 1 and the rest in
//    one shared accumulator.  Levels below NG - 1 are sums of at most
//    3 x 64 integer products below 2^16, hence integers below 2^24 and exact
//    whatever order and rounding the tensor core's FP32 adder uses;
//  * the slice count is chosen per item from the span of its matrix entries
//    (largest over smallest |entry|): NS = 4 (tile 128 x 32, NG = 3) while the
//    span is below 2^8, else NS = 6 (tile 128 x 16, NG = 4); dlogf items
//    always take six.  The per-row scale makes the error of a product grow
//    with the spread of magnitudes inside a row of L or a column of U: at
//    d = 3, Im k = -0.05, N = 1024 (span 2^6) four slices keep ln det within
//    ~1.4e-9 of FP64, while at d = 2, Im k = -0.3, N = 2048 (span 2^19, the
//    exponential growth e^{|Im k| r} over a disk of radius 25) they leave
//    ~1e-5 and six slices are needed;
//  * complex = 4 real products, Re uses the negate-B bit of the instruction
//    descriptor; the accumulators use 2 NG TN TMEM columns (192 or 128);
//  * epilogue: C (double-float, global) -= 2^(ea+eb-16) (sum of the levels).
// Operand slices are written to global images in the tensor core's
// core-matrix layout and moved to shared memory by bulk copies (TMA engine).
#include <cuda_bf16.h>
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include "engine_internal.h"
#include "lu64.cuh"
#include "df.cuh"
#include "umma.cuh"
#include "green_df.cuh"
#include "green_df2.cuh"

namespace msg {

constexpr int MT_M = 128;               // tile rows = TMEM lanes
constexpr int A_SUB = MT_M * NB * 2;    // one 128 x 32 bf16 operand tile: 8 KB
constexpr int TMEM_COLS = 256;          // accumulators: 2 NG TN <= 192 columns (allocation rounded to 2^k)
constexpr float RANGE_LIMIT = 1.0e18f;  // larger entries leave the safe FP32 exponent range
constexpr float SPAN_WIDE = 256.0f;     // entry span above which an item is sliced six ways
// amplitude items (iterative refinement to an FP64 residual): the LU only has to
// make the refinement contract, so four slices serve up to a far larger span
constexpr float SPAN_WIDE_REFINED = 1048576.0f;

// slice configurations: NS slices per operand, TN tile columns, NG TMEM accumulator groups
template <int NS> struct SliceCfg;
template <> struct SliceCfg<4> { static constexpr int TN = 32, NG = 3; };
template <> struct SliceCfg<6> { static constexpr int TN = 16, NG = 4; };
template <int NS> __host__ __device__ constexpr int a_band() { return 2 * NS * A_SUB; }  // NS slices x {Re, Im}
template <int NS> __host__ __device__ constexpr int b_sub() { return SliceCfg<NS>::TN * NB * 2; }
template <int NS> __host__ __device__ constexpr int b_band() { return 2 * NS * b_sub<NS>(); }
// shared-memory operand buffer: A band then B band (NS = 4: 64 + 16 KB; NS = 6: 96 + 12 KB)
constexpr int GEMM_BYTES = a_band<6>() + b_band<6>() > a_band<4>() + b_band<4>() ? a_band<6>() + b_band<6>()
                                                                                   : a_band<4>() + b_band<4>();
// global image bytes per 128 rows of A and per column of B, the larger of the two configurations
constexpr int A_IMG_BAND = a_band<6>();
constexpr int B_IMG_COL = b_band<6>() / SliceCfg<6>::TN > b_band<4>() / SliceCfg<4>::TN
                              ? b_band<6>() / SliceCfg<6>::TN : b_band<4>() / SliceCfg<4>::TN;

// per-phase cycle accounting (thread 0, only when X.stats is set)
enum { PH_ASSEMBLE = 0, PH_PANEL, PH_TRSM, PH_SLICE, PH_TILES, PH_SOLVE, PH_ITEMS, PH_N };

struct MixPanel {
    float4 T[NB][NB + 1];
    float4 T2[NB][NB + 1];
    float4 urow[NB];
    // assembly of d = 3 and d = 2: sin/cos/2^x tables, coordinates of the tile's atoms as
    // double-floats, and (d = 2) the item's K_nu constants
    Df3Tables tab;
    float4 ci[NB], cj[NB];  // x.h x.l y.h y.l
    float2 ciz[NB], cjz[NB];
    Df2Item d2;
    // assembly of d != 3: pair lists of the K_nu regime grouping
    unsigned short list[3 * 1024];
    int cnt[4];
};
struct MixGemm {
    uint8_t buf[GEMM_BYTES];  // A band at 0, B band at a_band<NS>()
};
// The operand buffers come last: a launch that never slices six ways (no item
// of its job can need it) allocates only the four-slice part of the union and
// leaves the rest of the SM's 256 KB of shared memory to the L1 cache.
struct MixSmem {
    uint64_t bar_a, bar_b, bar_mma;
    uint32_t tmem;
    int err;
    int mma_stuck;        // an MMA completion wait ran out: 1 + the parity it waited on
    zc diag[2];
    double red_v[NT / 32];
    int red_i[NT / 32];
    float red_f[NT / 32];
    double red_s[3][NT / 32];
    int info, bcast_i, item;
    unsigned long long stat[PH_N];
    long long t0;
    union alignas(128) {
        MixGemm g;
        MixPanel p;
    } u;
};
// dynamic shared memory of a launch with and without room for six slices
constexpr size_t MIX_SMEM_WIDE = sizeof(MixSmem) + 128;
constexpr size_t MIX_SMEM_NARROW =
    offsetof(MixSmem, u) + (sizeof(MixPanel) > (size_t)(a_band<4>() + b_band<4>()) ? sizeof(MixPanel)
                                                                                     : (size_t)(a_band<4>() + b_band<4>())) + 128;

__device__ __forceinline__ void stat_start(MixSmem& s) {
    if (threadIdx.x == 0) s.t0 = clock64();
}
__device__ __forceinline__ void stat_add(MixSmem& s, int ph) {
    if (threadIdx.x == 0) {
        long long t = clock64();
        s.stat[ph] += (unsigned long long)(t - s.t0);
        s.t0 = t;
    }
}

// per-CTA global scratch of the mixed engine
struct MixScratch {
    uint8_t* imgA;   // ceil(nmax/128) * A_IMG_BAND per CTA
    uint8_t* imgB;   // (ceil(nmax/32) * 32) * B_IMG_COL per CTA
    float* ea;       // row and column scales 2^(e-8) of the sliced operands, padded
    float* eb;
    size_t a_stride, b_stride, e_stride;
    int* err;        // device flag: 1 = an mbarrier wait timed out
    unsigned long long* stats;  // per-phase SM cycles summed over CTAs, or nullptr
    int first_wait;  // poll limit of the first operand wait of each trailing update (WAIT_LIMIT
                     // unless a test shortens it to make that wait run out)
};


struct Phases {
    uint32_t a, b, mma;
};

// ---------------------------------------------------------------- slicing
// NS pre-scaled bf16 slices of the double-float x (hi, lo) for row exponent e:
// x 2^(8-e) = s0 + s1 2^-9 + ... with integers |s_k| <= 256 (bf16 holds every
// integer up to 256 exactly); 8 + 9 (NS - 1) significant bits
template <int NS>
__device__ __forceinline__ void slice_n(float h, float l, int e, float* o) {
    float xh = ldexpf(h, 8 - e), xl = ldexpf(l, 8 - e);
    float s0 = rintf(xh);
    df r = two_sum(__fsub_rn(xh, s0), xl);
    o[0] = s0;
    float sc = 1.0f / 512.0f;
#pragma unroll
    for (int k = 1; k < NS; ++k) {
        float rh = __fmul_rn(r.h, 512.0f), rl = __fmul_rn(r.l, 512.0f);
        float sk = rintf(rh);
        r = two_sum(__fsub_rn(rh, sk), rl);
        o[k] = sk * sc;
        sc *= 1.0f / 512.0f;
    }
}

__device__ __forceinline__ int row_exponent(float mx) {
    int e = 0;
    if (mx > 0.0f) frexpf(mx, &e);
    return e;
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

// One operand row of K <= 32 complex values (stride `st` in float4) -> the
// 2 NS sub-tiles (slice k, Re/Im) of a band of R rows, row r; exponent returned.
template <int R, int NS>
__device__ __forceinline__ int slice_operand_row(const float4* __restrict__ src, size_t st, int K, uint8_t* band, int r) {
    float mx = 0.0f;
    for (int kk = 0; kk < K; ++kk) {
        float4 v = src[kk * st];
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.z)));
    }
    const int e = row_exponent(mx);
    constexpr int SUB = R * NB * 2;
    for (int kb = 0; kb < NB / 8; ++kb) {
        uint32_t w[2 * NS][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float re[2][NS], im[2][NS];
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const int kk = kb * 8 + 2 * q + t;
                if (kk < K) {
                    float4 v = src[kk * st];
                    slice_n<NS>(v.x, v.y, e, re[t]);
                    slice_n<NS>(v.z, v.w, e, im[t]);
                } else {
#pragma unroll
                    for (int sl = 0; sl < NS; ++sl) re[t][sl] = im[t][sl] = 0.0f;
                }
            }
#pragma unroll
            for (int sl = 0; sl < NS; ++sl) {
                w[2 * sl][q] = pack2(re[0][sl], re[1][sl]);
                w[2 * sl + 1][q] = pack2(im[0][sl], im[1][sl]);
            }
        }
        const uint32_t off = cm_offset(r, kb * 8, R);
#pragma unroll
        for (int sub = 0; sub < 2 * NS; ++sub)
            *reinterpret_cast<uint4*>(band + sub * SUB + off) = make_uint4(w[sub][0], w[sub][1], w[sub][2], w[sub][3]);
    }
    return e;
}

// A operand: rows [0, m) of the m x K panel P (column-major, ld), all bands;
// ea[i] = 2^(e_i - 8), the row's scale
template <int NS>
static __device__ void slice_panel_rows(const float4* __restrict__ P, int ld, int m, int K, uint8_t* img, float* ea) {
    const int mp = (m + MT_M - 1) / MT_M * MT_M;
    for (int i = threadIdx.x; i < mp; i += NT) {
        uint8_t* band = img + (size_t)(i / MT_M) * a_band<NS>();
        const int r = i % MT_M;
        if (i < m) {
            ea[i] = ldexpf(1.0f, slice_operand_row<MT_M, NS>(P + i, (size_t)ld, K, band, r) - 8);
        } else {
            ea[i] = 0.0f;
            for (int kb = 0; kb < NB / 8; ++kb)
                for (int sub = 0; sub < 2 * NS; ++sub)
                    *reinterpret_cast<uint4*>(band + sub * A_SUB + cm_offset(r, kb * 8, MT_M)) = make_uint4(0, 0, 0, 0);
        }
    }
}

// B operand: columns [0, nn) of the K x nn block Bp (column-major, ld); eb[j] = 2^(e_j - 8)
template <int NS>
static __device__ void slice_block_cols(const float4* __restrict__ Bp, int ld, int nn, int K, uint8_t* img, float* eb) {
    constexpr int TN = SliceCfg<NS>::TN;
    const int np = (nn + TN - 1) / TN * TN;
    for (int j = threadIdx.x; j < np; j += NT) {
        uint8_t* band = img + (size_t)(j / TN) * b_band<NS>();
        const int r = j % TN;
        if (j < nn) {
            eb[j] = ldexpf(1.0f, slice_operand_row<TN, NS>(Bp + (size_t)j * ld, 1, K, band, r) - 8);
        } else {
            eb[j] = 0.0f;
            for (int kb = 0; kb < NB / 8; ++kb)
                for (int sub = 0; sub < 2 * NS; ++sub)
                    *reinterpret_cast<uint4*>(band + sub * b_sub<NS>() + cm_offset(r, kb * 8, TN)) =
                        make_uint4(0, 0, 0, 0);
        }
    }
}

// ---------------------------------------------------------------- tensor-core update
// Accumulator group g (TMEM columns 2 TN g .. +TN for Re, +TN .. +2 TN for Im)
// holds slice level l = g for g < NG - 1 and levels >= NG - 1 in the last
// group, so that the low levels stay exact whatever the tensor core's FP32
// summation order and rounding.
template <int NS>
__device__ __forceinline__ void issue_tile_mmas(uint32_t a0, uint32_t b0, uint64_t* bar, uint32_t tmem) {
    constexpr int TN = SliceCfg<NS>::TN, NG = SliceCfg<NS>::NG, BSUB = b_sub<NS>();
    const uint32_t idp = idesc_bf16(MT_M, TN, false, false), idn = idesc_bf16(MT_M, TN, false, true);
    // core-matrix strides: K direction (LBO) R/8*128, row direction (SBO) 128; a K step of 16 is R*32 bytes
    auto dA = [&](int k, int c, int ks) { return sdesc(a0 + (k * 2 + c) * A_SUB + ks * (MT_M * 32), MT_M * 16, 128); };
    auto dB = [&](int k, int c, int ks) { return sdesc(b0 + (k * 2 + c) * BSUB + ks * (TN * 32), TN * 16, 128); };
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
#pragma unroll
        for (int l = 0; l < NS; ++l) {
            const int g = l < NG - 1 ? l : NG - 1;
#pragma unroll
            for (int i = 0; i <= l; ++i) {
                const int j = l - i;
                const uint32_t acc = (ks == 0 && i == 0 && l == g) ? 0u : 1u;  // first product of group g
                const uint32_t tre = tmem + 2 * TN * g, tim = tre + TN;
                umma_bf16(tre, dA(i, 0, ks), dB(j, 0, ks), idp, acc);
                umma_bf16(tre, dA(i, 1, ks), dB(j, 1, ks), idn, 1);
                umma_bf16(tim, dA(i, 0, ks), dB(j, 1, ks), idp, acc);
                umma_bf16(tim, dA(i, 1, ks), dB(j, 0, ks), idp, 1);
            }
        }
    }
    umma_commit(bar);
}

// c - (L0 + L1 + ... ): the exact levels enter by two-sums, the last group and
// every error term gather in one FP32 accumulator, one renormalisation
template <int NG>
__device__ __forceinline__ df df_sub_levels(df c, const float* lv) {
    df t = two_sum(c.h, -lv[0]);
    float lo = __fadd_rn(c.l, t.l);
#pragma unroll
    for (int g = 1; g < NG - 1; ++g) {
        const df u = two_sum(t.h, -lv[g]);
        lo = __fadd_rn(lo, u.l);
        t.h = u.h;
    }
    lo = __fsub_rn(lo, lv[NG - 1]);
    return quick_two_sum(t.h, lo);
}

// C[m x nn] -= Ap[m x K] * Bp[K x nn]; all double-float complex, column-major.
// tri != 0: only tiles holding an element with row >= column are updated.
// Returns false if a wait timed out (the engine then stops).
template <int NS>
static __device__ bool mixed_gemm_sub(float4* __restrict__ C, int ldc, const float4* __restrict__ Ap, int lda,
                               const float4* __restrict__ Bp, int ldb, int m, int nn, int K, int tri, MixSmem& s,
                               const MixScratch& X, uint32_t tmem, Phases& ph) {
    constexpr int TN = SliceCfg<NS>::TN, NG = SliceCfg<NS>::NG, AB = a_band<NS>(), BB = b_band<NS>();
    constexpr int CW = TN / 2;  // columns of a tile per thread (two warps per TMEM lane quadrant)
    if (m <= 0 || nn <= 0 || K <= 0) return true;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t* imgA = X.imgA + (size_t)blockIdx.x * X.a_stride;
    uint8_t* imgB = X.imgB + (size_t)blockIdx.x * X.b_stride;
    float* gea = X.ea + (size_t)blockIdx.x * X.e_stride;
    float* geb = X.eb + (size_t)blockIdx.x * X.e_stride;
    uint8_t* sA = s.u.g.buf;
    uint8_t* sB = s.u.g.buf + AB;
    stat_start(s);
    slice_panel_rows<NS>(Ap, lda, m, K, imgA, gea);
    slice_block_cols<NS>(Bp, ldb, nn, K, imgB, geb);
    fence_proxy_async_all();
    __syncthreads();
    stat_add(s, PH_SLICE);
    const int nbi = (m + MT_M - 1) / MT_M, nbj = (nn + TN - 1) / TN;
    // tile list in row-band order, skipping tiles wholly above the diagonal when tri
    auto tile_ok = [&](int bi, int bj) { return !tri || bi * MT_M + MT_M - 1 >= bj * TN; };
    auto next_tile = [&](int& bi, int& bj) {
        do {
            if (++bj >= nbj) { bj = 0; ++bi; }
        } while (bi < nbi && !tile_ok(bi, bj));
    };
    int bi = 0, bj = 0;
    if (!tile_ok(bi, bj)) next_tile(bi, bj);
    if (bi >= nbi) return true;
    if (tid == 0) {
        mbar_arrive_expect_tx(&s.bar_a, AB);
        bulk_g2s(sA, imgA + (size_t)bi * AB, AB / 2, &s.bar_a);
        bulk_g2s(sA + AB / 2, imgA + (size_t)bi * AB + AB / 2, AB / 2, &s.bar_a);
        mbar_arrive_expect_tx(&s.bar_b, BB);
        bulk_g2s(sB, imgB + (size_t)bj * BB, BB, &s.bar_b);
    }
    bool ok = true;
    bool new_band = true, first = true;
    const int q = warp & 3, hcol = warp >> 2;  // TMEM lane quadrant, column half of this warp
    const int rloc = 32 * q + lane;
    while (bi < nbi) {
        int nbi2 = bi, nbj2 = bj;
        next_tile(nbi2, nbj2);
        // this thread's row and CW columns of C, and its row scale, fetched before
        // the MMAs complete so the memory latency hides behind the tensor core
        const int row = bi * MT_M + rloc;
        const bool row_ok = row < m;
        const float ea_r = row_ok ? gea[row] : 0.0f;
        float4 cpre[CW];
#pragma unroll
        for (int j = 0; j < CW; ++j) {
            const int col = bj * TN + CW * hcol + j;
            cpre[j] = (row_ok && col < nn) ? C[row + (size_t)col * ldc] : make_float4(0, 0, 0, 0);
        }
        if (tid == 0) {
            bool w = true;
            if (new_band) {
                w = mbar_wait(&s.bar_a, ph.a, first ? X.first_wait : WAIT_LIMIT);
                if (!w) mbar_wait(&s.bar_a, ph.a);  // let the copy in flight land before moving on
                ph.a ^= 1;
            }
            const bool wb = mbar_wait(&s.bar_b, ph.b);
            ph.b ^= 1;
            if (w && wb) {
                tc_fence_after();
                issue_tile_mmas<NS>(smem_u32(sA), smem_u32(sB), &s.bar_mma, tmem);
            } else {
                s.err = 1;                // operands missing: no MMA is issued, the CTA stops
                mbar_arrive(&s.bar_mma);  // after this tile; release its MMA wait at once
            }
        }
        first = false;
        const bool mw = mbar_wait(&s.bar_mma, ph.mma);
        if (!mw && lane == 0) {
            s.err = 1;
            s.mma_stuck = 1 + (int)ph.mma;
        }
        ph.mma ^= 1;
        // operands of the next tile: smem is free once the MMAs completed (none after a failed wait)
        if (tid == 0 && nbi2 < nbi && !s.err) {
            if (nbi2 != bi) {
                mbar_arrive_expect_tx(&s.bar_a, AB);
                bulk_g2s(sA, imgA + (size_t)nbi2 * AB, AB / 2, &s.bar_a);
                bulk_g2s(sA + AB / 2, imgA + (size_t)nbi2 * AB + AB / 2, AB / 2, &s.bar_a);
            }
            mbar_arrive_expect_tx(&s.bar_b, BB);
            bulk_g2s(sB, imgB + (size_t)nbj2 * BB, BB, &s.bar_b);
        }
        tc_fence_after();
        // epilogue: TMEM lanes 32(w%4).. (rows), columns CW(w/4)..+CW-1
#pragma unroll
        for (int cc = 0; cc < CW; cc += 4) {
            float g[2 * NG][4];
            const uint32_t base = tmem + ((uint32_t)(32 * q) << 16) + CW * hcol + cc;
#pragma unroll
            for (int a = 0; a < 2 * NG; ++a) tmem_ld4(base + TN * a, g[a]);
            tmem_wait_ld();
            if (row_ok) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int col = bj * TN + CW * hcol + cc + j;
                    if (col < nn) {
                        const float sc = ea_r * __ldg(geb + col);  // 2^(ea+eb-16), exact
                        const float4 cv = cpre[cc + j];
                        dfc c = dfc{df{cv.x, cv.y}, df{cv.z, cv.w}};
                        float lr[NG], li[NG];
#pragma unroll
                        for (int gg = 0; gg < NG; ++gg) {
                            lr[gg] = g[2 * gg][j] * sc;
                            li[gg] = g[2 * gg + 1][j] * sc;
                        }
                        c.re = df_sub_levels<NG>(c.re, lr);
                        c.im = df_sub_levels<NG>(c.im, li);
                        dfc_store(C + row + (size_t)col * ldc, c);
                    }
                }
            }
        }
        tc_fence_before();
        __syncthreads();
        new_band = (nbi2 != bi);
        bi = nbi2;
        bj = nbj2;
        if (s.err) {
            ok = false;
            break;
        }
    }
    stat_add(s, PH_TILES);
    return ok;
}

// ---------------------------------------------------------------- double-float panel, TRSM, solves
// arg max of v over the CTA (smallest index on ties), in FP32: the FP64 pipe
// (1/64 of the FP32 rate on GB300) stays out of the panel's per-column steps
__device__ __forceinline__ int block_argmaxf(float v, int i, MixSmem& s) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float v2 = __shfl_down_sync(FULL, v, off);
        const int i2 = __shfl_down_sync(FULL, i, off);
        if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
    }
    if (lane == 0) { s.red_f[warp] = v; s.red_i[warp] = i; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float bv = s.red_f[0];
        int bi = s.red_i[0];
        for (int w = 1; w < NT / 32; w++) {
            const float v2 = s.red_f[w];
            const int i2 = s.red_i[w];
            if (v2 > bv || (v2 == bv && i2 < bi)) { bv = v2; bi = i2; }
        }
        s.bcast_i = bi;
    }
    __syncthreads();
    return s.bcast_i;
}

// 1 / b in double-float, with b scaled by a power of two first so that its
// squared modulus stays inside the FP32 range whatever the pivot's size
__device__ __forceinline__ dfc dfc_recip_pow2(dfc b) {
    int e;
    frexpf(fmaxf(fabsf(b.re.h), fabsf(b.im.h)), &e);
    const float sc = ldexpf(1.0f, -e);
    const dfc r = dfc_recip(dfc{df{b.re.h * sc, b.re.l * sc}, df{b.im.h * sc, b.im.l * sc}});
    return dfc{df{r.re.h * sc, r.re.l * sc}, df{r.im.h * sc, r.im.l * sc}};
}

// Panel factorisation in double-float: LAPACK's getf2 pivoting (|Re|+|Im|,
// first index on ties, full-panel row interchanges), organised in sub-panels
// of SW columns.  Inside a sub-panel the rank-1 updates touch only its own
// columns; the rest of the panel then takes one rank-SW update per sub-panel
// (U rows by unit-lower substitution in shared memory).  The panel of a large
// matrix does not stay in L2 across 304 resident CTAs, so this cuts its
// memory traffic (the full-width rank-1 form re-reads and re-writes the whole
// remaining panel once per column) by about 2.4x at the same arithmetic.
// The pivot's reciprocal is a double-float one that every thread computes
// (the FP64 division by one thread, on a pipe at 1/64 of the FP32 rate, held
// the whole CTA at the next barrier).
// Not inlined: its registers are then allocated apart from the engine's
// tensor-core epilogue, which holds the kernel at the 128-register cap.
constexpr int SW = 4;

static __device__ __noinline__ void df_panel(float4* __restrict__ A, int n, int j0, int jb, int* __restrict__ ipiv, MixSmem& s) {
    const int tid = threadIdx.x;
    const int cend = j0 + jb;
    float bv = -1.0f;
    int bi = n;
    for (int i = j0 + tid; i < n; i += NT) {
        const float v = dfc_abs1(dfc_load(A + i + (size_t)j0 * n));
        if (v > bv) { bv = v; bi = i; }
    }
    for (int c0 = j0; c0 < cend; c0 += SW) {
        const int sw = min(c0 + SW, cend);  // sub-panel columns [c0, sw)
        for (int c = c0; c < sw; ++c) {
            int p = block_argmaxf(bv, bi, s);
            if (p >= n) p = c;
            const dfc piv = dfc_load(A + p + (size_t)c * n);
            const bool nz = !dfc_is_zero(piv);
            if (tid == 0) {
                ipiv[c] = p;
                if (!nz && s.info == 0) s.info = c + 1;
            }
            const dfc r = nz ? dfc_recip_pow2(piv) : dfc{df{0, 0}, df{0, 0}};
            __syncthreads();  // every thread holds the pivot before row p is swapped away
            if (nz && p != c && tid < jb) {
                const size_t col = (size_t)(j0 + tid) * n;
                float4 t = A[c + col];
                A[c + col] = A[p + col];
                A[p + col] = t;
            }
            __syncthreads();
            if (tid < jb && j0 + tid > c && j0 + tid < sw) s.u.p.urow[tid] = A[c + (size_t)(j0 + tid) * n];
            __syncthreads();
            bv = -1.0f;
            bi = n;
            if (nz) {
                for (int i = c + 1 + tid; i < n; i += NT) {
                    float4* pc = A + i + (size_t)c * n;
                    const dfc l = dfc_mul(dfc_load(pc), r);
                    dfc_store(pc, l);
                    if (c + 1 < sw) {
                        float4* q1 = A + i + (size_t)(c + 1) * n;
                        const dfc a = dfc_fms(dfc_load(q1), l, dfc_load(&s.u.p.urow[c + 1 - j0]));
                        dfc_store(q1, a);
                        const float v = dfc_abs1(a);
                        if (v > bv) { bv = v; bi = i; }
                        for (int cc = c + 2; cc < sw; ++cc) {
                            float4* qp = A + i + (size_t)cc * n;
                            dfc_store(qp, dfc_fms(dfc_load(qp), l, dfc_load(&s.u.p.urow[cc - j0])));
                        }
                    }
                }
            } else if (c + 1 < sw) {
                for (int i = c + 1 + tid; i < n; i += NT) {
                    const float v = dfc_abs1(dfc_load(A + i + (size_t)(c + 1) * n));
                    if (v > bv) { bv = v; bi = i; }
                }
            }
        }
        if (sw < cend) {
            const int cw = sw - c0, rem = cend - sw;
            __syncthreads();  // the sub-panel's last column is complete
            // L11 (unit lower, cw x cw) into shared memory
            if (tid < cw * cw) {
                const int r = tid / cw, q = tid % cw;
                if (q < r) s.u.p.T2[r][q] = A[c0 + r + (size_t)(c0 + q) * n];
            }
            __syncthreads();
            // U rows of the sub-panel for columns [sw, cend): u_r = a_r - sum_{q<r} L_rq u_q
            if (tid < rem) {
                const size_t col = (size_t)(sw + tid) * n;
                dfc u[SW];
#pragma unroll
                for (int r = 0; r < SW; ++r) {
                    if (r < cw) {
                        dfc a = dfc_load(A + c0 + r + col);
#pragma unroll
                        for (int q = 0; q < r; ++q) a = dfc_fms(a, dfc_load(&s.u.p.T2[r][q]), u[q]);
                        u[r] = a;
                        dfc_store(A + c0 + r + col, a);
                        dfc_store(&s.u.p.T[r][tid], a);
                    }
                }
            }
            __syncthreads();
            // rank-cw update of rows >= sw; argmax of column sw on the way
            bv = -1.0f;
            bi = n;
            for (int i = sw + tid; i < n; i += NT) {
                dfc l[SW];
#pragma unroll
                for (int q = 0; q < SW; ++q)
                    if (q < cw) l[q] = dfc_load(A + i + (size_t)(c0 + q) * n);
                for (int t = 0; t < rem; ++t) {
                    float4* qp = A + i + (size_t)(sw + t) * n;
                    dfc a = dfc_load(qp);
#pragma unroll
                    for (int q = 0; q < SW; ++q)
                        if (q < cw) a = dfc_fms(a, l[q], dfc_load(&s.u.p.T[q][t]));
                    dfc_store(qp, a);
                    if (t == 0) {
                        const float v = dfc_abs1(a);
                        if (v > bv) { bv = v; bi = i; }
                    }
                }
            }
        }
    }
    __syncthreads();
}

__device__ __forceinline__ void dcol_lower_unit(float4* __restrict__ b, int jb, const float4 (*T)[NB + 1]) {
    for (int rb = 0; rb < jb; rb += CH) {
        dfc y[CH];
#pragma unroll
        for (int r = 0; r < CH; ++r) y[r] = (rb + r < jb) ? dfc_load(b + rb + r) : dfc{df{0, 0}, df{0, 0}};
        for (int q = 0; q < rb; ++q) {
            const dfc xq = dfc_load(b + q);
#pragma unroll
            for (int r = 0; r < CH; ++r) y[r] = dfc_fms(y[r], dfc_load(&T[rb + r][q]), xq);
        }
#pragma unroll
        for (int r = 1; r < CH; ++r)
#pragma unroll
            for (int q = 0; q < r; ++q) y[r] = dfc_fms(y[r], dfc_load(&T[rb + r][rb + q]), y[q]);
#pragma unroll
        for (int r = 0; r < CH; ++r)
            if (rb + r < jb) dfc_store(b + rb + r, y[r]);
    }
}

// upper solve; T's diagonal holds the reciprocals of U_rr
__device__ __forceinline__ void dcol_upper(float4* __restrict__ b, int jb, const float4 (*T)[NB + 1]) {
    for (int rb = ((jb - 1) / CH) * CH; rb >= 0; rb -= CH) {
        dfc y[CH];
#pragma unroll
        for (int r = 0; r < CH; ++r) y[r] = (rb + r < jb) ? dfc_load(b + rb + r) : dfc{df{0, 0}, df{0, 0}};
        for (int q = rb + CH; q < jb; ++q) {
            const dfc xq = dfc_load(b + q);
#pragma unroll
            for (int r = 0; r < CH; ++r) y[r] = dfc_fms(y[r], dfc_load(&T[rb + r][q]), xq);
        }
#pragma unroll
        for (int r = CH - 1; r >= 0; --r) {
            if (rb + r < jb) {
                dfc acc = y[r];
#pragma unroll
                for (int q = r + 1; q < CH; ++q) acc = dfc_fms(acc, dfc_load(&T[rb + r][rb + q]), y[q]);
                y[r] = dfc_mul(acc, dfc_load(&T[rb + r][rb + r]));
            }
        }
#pragma unroll
        for (int r = 0; r < CH; ++r)
            if (rb + r < jb) dfc_store(b + rb + r, y[r]);
    }
}

static __device__ void load_lower_block(const float4* A, int n, int j0, int jb, MixSmem& s) {
    for (int e = threadIdx.x; e < NB * NB; e += NT) {
        int r = e % NB, q = e / NB;
        s.u.p.T[r][q] = (r < jb && q < r) ? A[(j0 + r) + (size_t)(j0 + q) * n] : make_float4(0, 0, 0, 0);
    }
    __syncthreads();
}

static __device__ void load_upper_block(const float4* A, int n, int j0, int jb, MixSmem& s) {
    for (int e = threadIdx.x; e < NB * NB; e += NT) {
        int r = e % NB, q = e / NB;
        float4 v = make_float4(0, 0, 0, 0);
        if (r < jb && q < jb && q > r) v = A[(j0 + r) + (size_t)(j0 + q) * n];
        if (r == q) {
            if (r < jb) {
                const dfc u = dfc_load(A + (j0 + r) + (size_t)(j0 + r) * n);
                const zc ri = 1.0 / mk(df_to_double(u.re), df_to_double(u.im));
                const df a = df_from_double(ri.re), b = df_from_double(ri.im);
                v = make_float4(a.h, a.l, b.h, b.l);
            } else {
                v = make_float4(1, 0, 0, 0);
            }
        }
        s.u.p.T[r][q] = v;
    }
    __syncthreads();
}

// The panel's row interchanges on the columns outside it, then the TRSM
// U12 = L11^-1 A12 of the columns right of it.  keep_l = false leaves the columns
// left of the panel alone: a ln det reads only U's diagonal and the pivots.
static __device__ void df_swaps_trsm(float4* __restrict__ A, int n, int j0, int jb, const int* __restrict__ ipiv,
                                     MixSmem& s, bool keep_l) {
    load_lower_block(A, n, j0, jb, s);
    for (int col = keep_l ? threadIdx.x : j0 + threadIdx.x; col < n; col += NT) {
        if (col >= j0 && col < j0 + jb) continue;
        float4* a = A + (size_t)col * n;
        for (int c = j0; c < j0 + jb; ++c) {
            int p = ipiv[c];
            if (p != c) { float4 t = a[c]; a[c] = a[p]; a[p] = t; }
        }
        if (col >= j0 + jb) dcol_lower_unit(a + j0, jb, s.u.p.T);
    }
    __syncthreads();
}

template <int NS>
static __device__ bool lu_mixed(float4* __restrict__ A, int n, int* __restrict__ ipiv, bool keep_l, MixSmem& s,
                                const MixScratch& X, uint32_t tmem, Phases& ph) {
    for (int j0 = 0; j0 < n; j0 += NB) {
        const int jb = min(NB, n - j0);
        stat_start(s);
        df_panel(A, n, j0, jb, ipiv, s);
        stat_add(s, PH_PANEL);
        df_swaps_trsm(A, n, j0, jb, ipiv, s, keep_l);
        stat_add(s, PH_TRSM);
        const int r0 = j0 + jb;
        if (!mixed_gemm_sub<NS>(A + r0 + (size_t)r0 * n, n, A + r0 + (size_t)j0 * n, n, A + j0 + (size_t)r0 * n, n,
                            n - r0, n - r0, jb, 0, s, X, tmem, ph))
            return false;
    }
    return true;
}

// tr(A^-1 B) from the mixed LU of A; B (double-float, n x n) is destroyed
template <int NS>
static __device__ bool trace_solve_mixed(const float4* __restrict__ A, float4* __restrict__ B, int n,
                                  const int* __restrict__ ipiv, MixSmem& s, const MixScratch& X, uint32_t tmem,
                                  Phases& ph, zc& out) {
    const int tid = threadIdx.x;
    for (int col = tid; col < n; col += NT) {
        float4* b = B + (size_t)col * n;
        for (int i = 0; i < n; ++i) {
            int p = ipiv[i];
            if (p != i) { float4 t = b[i]; b[i] = b[p]; b[p] = t; }
        }
    }
    __syncthreads();
    for (int j0 = 0; j0 < n; j0 += NB) {
        const int jb = min(NB, n - j0);
        load_lower_block(A, n, j0, jb, s);
        for (int col = tid; col < n; col += NT) dcol_lower_unit(B + (size_t)col * n + j0, jb, s.u.p.T);
        __syncthreads();
        const int r0 = j0 + jb;
        if (!mixed_gemm_sub<NS>(B + r0, n, A + r0 + (size_t)j0 * n, n, B + j0, n, n - r0, n, jb, 0, s, X, tmem, ph))
            return false;
    }
    const int nblk = (n + NB - 1) / NB;
    for (int kb = nblk - 1; kb >= 0; --kb) {
        const int j0 = kb * NB, jb = min(NB, n - j0), ncol = j0 + jb;
        load_upper_block(A, n, j0, jb, s);
        for (int col = tid; col < ncol; col += NT) dcol_upper(B + (size_t)col * n + j0, jb, s.u.p.T);
        __syncthreads();
        if (!mixed_gemm_sub<NS>(B, n, A + (size_t)j0 * n, n, B + j0, n, j0, ncol, jb, 1, s, X, tmem, ph)) return false;
    }
    double tr = 0.0, ti = 0.0, z = 0.0;
    for (int i = tid; i < n; i += NT) {
        dfc v = dfc_load(B + i + (size_t)i * n);
        tr += df_to_double(v.re);
        ti += df_to_double(v.im);
    }
    block_sum3(tr, ti, z, s);
    out = mk(tr, ti);
    return true;
}

// (largest, smallest non-zero) of max(|Re|, |Im|) over the entries seen, with v added
__device__ __forceinline__ float2 entry_range(float2 rg, float4 v) {
    const float a = fmaxf(fabsf(v.x), fabsf(v.z));
    return make_float2(fmaxf(rg.x, a), a > 0.0f ? fminf(rg.y, a) : rg.y);
}

// One 32 x 32 tile of a d != 3 matrix (K_nu elements, FP64, grouped by regime)
// stored as double-floats: the direct triangle here, the mirror by the caller.
// Not inlined, so that d = 3 matrices keep the kernel's registers for themselves.
// rg: the largest and the smallest non-zero max(|Re|, |Im|) of the entries seen.
static __device__ __noinline__ float2 assemble_tile_grouped(float4* __restrict__ A, float4* __restrict__ B, int n,
                                                    int d, const double* __restrict__ pos, zc k, int I, int J,
                                                    zc dg0, zc dg1, MixSmem& s, float2 rg) {
    const int tid = threadIdx.x;
    auto cvt = [](zc v) {
        df a = df_from_double(v.re), b = df_from_double(v.im);
        return make_float4(a.h, a.l, b.h, b.l);
    };
    tile_pairs_grouped(I, J, n, d, pos, k, B != nullptr, s.u.p.list, s.u.p.cnt, [&](int ii, int jj, zc m, zc dm) {
        const float4 fm = cvt(m);
        rg = entry_range(rg, fm);
        s.u.p.T[jj][ii] = fm;
        if (B) {
            const float4 fd = cvt(dm);
            rg = entry_range(rg, fd);
            s.u.p.T2[jj][ii] = fd;
        }
    });
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ii = tid & 31, jj = (tid >> 5) + 8 * q;
        const int i = I * 32 + ii, j = J * 32 + jj;
        if (i < n && j < n && i <= j) {
            float4 fm = s.u.p.T[jj][ii], fd = make_float4(0, 0, 0, 0);
            if (B) fd = s.u.p.T2[jj][ii];
            if (i == j) {
                fm = cvt(dg0);
                rg = entry_range(rg, fm);
                if (B) {
                    fd = cvt(dg1);
                    rg = entry_range(rg, fd);
                }
            }
            A[i + (size_t)j * n] = fm;
            if (B) B[i + (size_t)j * n] = fd;
        }
    }
    return rg;
}

// One 32 x 32 tile of a d = 2 matrix, every element on the FP32 pipe in
// double-float (green_df2.cuh), the pairs grouped by K_nu regime as in the
// FP64 engine (tile_pairs_grouped): classified into three shared-memory lists,
// then consecutive threads take consecutive list entries, so that a warp runs
// one regime's loop.  Direct triangle here, the mirror by the caller.
static __device__ __noinline__ float2 assemble_tile_grouped_df2(float4* __restrict__ A, float4* __restrict__ B, int n,
                                                        int I, int J, zc dg0, zc dg1, MixSmem& s, float2 rg) {
    const int tid = threadIdx.x;
    const Df2Item& P = s.u.p.d2;
    unsigned short* list = s.u.p.list;
    int* cnt = s.u.p.cnt;
    auto dist = [&](int ii, int jj) {
        const float4 pa = s.u.p.ci[ii], pb = s.u.p.cj[jj];
        const df ex = df_sub(df{pa.x, pa.y}, df{pb.x, pb.y});
        const df ey = df_sub(df{pa.z, pa.w}, df{pb.z, pb.w});
        return df_sqrt(df_add(df_mul(ex, ex), df_mul(ey, ey)));
    };
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int p = tid + NT * q, ii = p & 31, jj = p >> 5;
        const int i = I * 32 + ii, j = J * 32 + jj;
        if (i < n && j < n && i < j) {
            const int reg = k_regime_df(P, dist(ii, jj));
            list[reg * 1024 + atomicAdd(&cnt[reg], 1)] = (unsigned short)p;
        }
    }
    __syncthreads();
    const int c0 = cnt[0], c1 = cnt[1], tot = c0 + c1 + cnt[2];
    for (int w = tid; w < tot; w += NT) {
        const int reg = w < c0 ? 0 : (w < c0 + c1 ? 1 : 2);
        const int p = reg == 0 ? list[w] : (reg == 1 ? list[1024 + w - c0] : list[2048 + w - c0 - c1]);
        const int ii = p & 31, jj = p >> 5;
        dfc m, dm;
        pair_elements_df2(s.u.p.tab, P, dist(ii, jj), reg, B != nullptr, m, dm);
        const float4 fm = make_float4(m.re.h, m.re.l, m.im.h, m.im.l);
        rg = entry_range(rg, fm);
        s.u.p.T[jj][ii] = fm;
        if (B) {
            const float4 fd = make_float4(dm.re.h, dm.re.l, dm.im.h, dm.im.l);
            rg = entry_range(rg, fd);
            s.u.p.T2[jj][ii] = fd;
        }
    }
    __syncthreads();
    if (tid < 3) cnt[tid] = 0;
    auto cvt = [](zc v) {
        df a = df_from_double(v.re), b = df_from_double(v.im);
        return make_float4(a.h, a.l, b.h, b.l);
    };
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int ii = tid & 31, jj = (tid >> 5) + 8 * q;
        const int i = I * 32 + ii, j = J * 32 + jj;
        if (i < n && j < n && i <= j) {
            float4 fm = s.u.p.T[jj][ii], fd = make_float4(0, 0, 0, 0);
            if (B) fd = s.u.p.T2[jj][ii];
            if (i == j) {
                fm = cvt(dg0);
                rg = entry_range(rg, fm);
                if (B) {
                    fd = cvt(dg1);
                    rg = entry_range(rg, fd);
                }
            }
            A[i + (size_t)j * n] = fm;
            if (B) B[i + (size_t)j * n] = fd;
        }
    }
    return rg;
}

// Assembly of M(k) (and dM/dk into B) as double-floats; returns the largest
// and the smallest non-zero max(|Re|, |Im|) over the entries this thread stored.
template <bool D3ONLY>
__device__ float2 assemble_df(float4* __restrict__ A, float4* __restrict__ B, int n, int d,
                             const double* __restrict__ pos, const msgpu_model& mdl, zc k, MixSmem& s) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        s.diag[0] = invf(mdl, d, k);
        if (B) s.diag[1] = dk_invf(mdl, d, k);
    }
    __syncthreads();
    const zc dg0 = s.diag[0], dg1 = s.diag[1];
    const bool d3 = D3ONLY || d == 3;
    const df kr = df_from_double(k.re), ki = df_from_double(k.im);
    const bool grow = k.im != 0.0;
    const bool grouped = !D3ONLY && d != 3 && d != 1;
    const bool d2 = !D3ONLY && d == 2;  // d = 2: every element on the FP32 pipe too (green_df2.cuh)
    if (d3 || d2) df3_tables_init(s.u.p.tab);
    if (d2 && tid == 0) s.u.p.d2 = df2_item(k);
    if (grouped && tid < 3) s.u.p.cnt[tid] = 0;
    __syncthreads();
    float2 rg = make_float2(0.0f, INFINITY);
    auto cvt = [](zc v) {
        df a = df_from_double(v.re), b = df_from_double(v.im);
        return make_float4(a.h, a.l, b.h, b.l);
    };
    const int nt = (n + 31) / 32;
    for (int J = 0; J < nt; ++J) {
        for (int I = 0; I <= J; ++I) {
            if (d3 || d2) {
                // the tile's atoms as double-floats: rows I*32.., columns J*32..
                if (tid < 64) {
                    const int a = (tid < 32 ? I : J) * 32 + (tid & 31);
                    const int dd = d3 ? 3 : 2;
                    df x{0.0f, 0.0f}, y{0.0f, 0.0f}, z{0.0f, 0.0f};
                    if (a < n) {
                        x = df_from_double(pos[dd * a]);
                        y = df_from_double(pos[dd * a + 1]);
                        if (d3) z = df_from_double(pos[3 * a + 2]);
                    }
                    if (tid < 32) {
                        s.u.p.ci[tid] = make_float4(x.h, x.l, y.h, y.l);
                        s.u.p.ciz[tid] = make_float2(z.h, z.l);
                    } else {
                        s.u.p.cj[tid - 32] = make_float4(x.h, x.l, y.h, y.l);
                        s.u.p.cjz[tid - 32] = make_float2(z.h, z.l);
                    }
                }
                __syncthreads();
            }
            if (grouped) {
                rg = d2 ? assemble_tile_grouped_df2(A, B, n, I, J, dg0, dg1, s, rg)
                        : assemble_tile_grouped(A, B, n, d, pos, k, I, J, dg0, dg1, s, rg);
            } else {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int ii = tid & 31, jj = (tid >> 5) + 8 * q;
                    const int i = I * 32 + ii, j = J * 32 + jj;
                    if (i < n && j < n && i <= j) {
                        float4 fm, fd = make_float4(0, 0, 0, 0);
                        if (i < j && d3) {
                            // the whole element on the FP32 pipe in double-float (green_df.cuh)
                            const float4 pa = s.u.p.ci[ii], pb = s.u.p.cj[jj];
                            const float2 za = s.u.p.ciz[ii], zb = s.u.p.cjz[jj];
                            const df ex = df_sub(df{pa.x, pa.y}, df{pb.x, pb.y});
                            const df ey = df_sub(df{pa.z, pa.w}, df{pb.z, pb.w});
                            const df ez = df_sub(df{za.x, za.y}, df{zb.x, zb.y});
                            const df r = df_sqrt(df_add(df_add(df_mul(ex, ex), df_mul(ey, ey)), df_mul(ez, ez)));
                            dfc a, b;
                            pair_elements_df3t(s.u.p.tab, kr, ki, grow, r, B != nullptr, a, b);
                            fm = make_float4(a.re.h, a.re.l, a.im.h, a.im.l);
                            if (B) fd = make_float4(b.re.h, b.re.l, b.im.h, b.im.l);
                        } else {
                            zc m, dm = mk(0.0);
                            if (i < j) {
                                pair_elements(d, k, atom_distance(d, pos, i, j), B != nullptr, m, dm);
                            } else {
                                m = dg0;
                                dm = dg1;
                            }
                            fm = cvt(m);
                            if (B) fd = cvt(dm);
                        }
                        rg = entry_range(rg, fm);
                        A[i + (size_t)j * n] = fm;
                        s.u.p.T[jj][ii] = fm;
                        if (B) {
                            rg = entry_range(rg, fd);
                            B[i + (size_t)j * n] = fd;
                            s.u.p.T2[jj][ii] = fd;
                        }
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int jj = tid & 31, ii = (tid >> 5) + 8 * q;
                const int i = I * 32 + ii, j = J * 32 + jj;
                if (j < n && i < j) {
                    A[j + (size_t)i * n] = s.u.p.T[jj][ii];
                    if (B) B[j + (size_t)i * n] = s.u.p.T2[jj][ii];
                }
            }
            __syncthreads();
        }
    }
    return rg;
}

// after block_argmax: the CTA-wide maximum (thread 0 folded the warp maxima into red_v)
__device__ __forceinline__ double block_max_value(MixSmem& s) {
    double m = s.red_v[0];
    for (int w = 1; w < NT / 32; ++w) m = fmax(m, s.red_v[w]);
    return m;
}

static __device__ zc tracelog_df(const float4* __restrict__ A, int n, const int* __restrict__ ipiv, MixSmem& s) {
    double lr = 0.0, ar = 0.0, odd = 0.0;
    for (int i = threadIdx.x; i < n; i += NT) {
        const dfc u = dfc_load(A + i + (size_t)i * n);
        const double re = df_to_double(u.re), im = df_to_double(u.im);
        lr += log(hypot(re, im));
        ar += atan2(im, re);
        if (ipiv[i] != i) odd += 1.0;
    }
    block_sum3(lr, ar, odd, s);
    if (fmod(odd, 2.0) == 1.0) ar += PI;
    return mk(lr / n, ar / n);
}

// x <- (LU)^-1 x, one right-hand side, double-float (LAPACK-layout LU): the
// interchanges, then blocked substitution; each block's triangle by warp 0
// (one row per lane), the rectangular part by all threads (one row each)
static __device__ void df_solve_vec(const float4* __restrict__ A, float4* __restrict__ x, int n,
                             const int* __restrict__ ipiv, MixSmem& s) {
    const unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0)
        for (int i = 0; i < n; ++i) {
            int p = ipiv[i];
            if (p != i) { float4 t = x[i]; x[i] = x[p]; x[p] = t; }
        }
    __syncthreads();
    auto shfl4 = [&](float4 v, int src) {
        return make_float4(__shfl_sync(FULL, v.x, src), __shfl_sync(FULL, v.y, src), __shfl_sync(FULL, v.z, src),
                           __shfl_sync(FULL, v.w, src));
    };
    for (int j0 = 0; j0 < n; j0 += NB) {
        const int jb = min(NB, n - j0);
        if (tid < 32) {
            float4 v = lane < jb ? x[j0 + lane] : make_float4(0, 0, 0, 0);
            for (int q = 0; q < jb - 1; ++q) {
                const float4 xq = shfl4(v, q);
                if (lane > q && lane < jb) {
                    dfc r = dfc_fms(dfc{df{v.x, v.y}, df{v.z, v.w}}, dfc_load(A + (j0 + lane) + (size_t)(j0 + q) * n),
                                    dfc{df{xq.x, xq.y}, df{xq.z, xq.w}});
                    v = make_float4(r.re.h, r.re.l, r.im.h, r.im.l);
                }
            }
            if (lane < jb) x[j0 + lane] = v;
        }
        __syncthreads();
        for (int i = j0 + jb + tid; i < n; i += NT) {
            dfc acc = dfc_load(x + i);
            for (int q = 0; q < jb; ++q) acc = dfc_fms(acc, dfc_load(A + i + (size_t)(j0 + q) * n), dfc_load(x + j0 + q));
            dfc_store(x + i, acc);
        }
        __syncthreads();
    }
    const int nblk = (n + NB - 1) / NB;
    for (int kb = nblk - 1; kb >= 0; --kb) {
        const int j0 = kb * NB, jb = min(NB, n - j0);
        if (tid < 32) {
            float4 v = lane < jb ? x[j0 + lane] : make_float4(0, 0, 0, 0);
            for (int q = jb - 1; q >= 0; --q) {
                if (lane == q) {
                    const dfc u = dfc_load(A + (j0 + q) + (size_t)(j0 + q) * n);
                    const zc xv = mk(df_to_double(df{v.x, v.y}), df_to_double(df{v.z, v.w}));
                    const zc qv = xv / mk(df_to_double(u.re), df_to_double(u.im));
                    const df a = df_from_double(qv.re), b = df_from_double(qv.im);
                    v = make_float4(a.h, a.l, b.h, b.l);
                }
                const float4 xq = shfl4(v, q);
                if (lane < q) {
                    dfc r = dfc_fms(dfc{df{v.x, v.y}, df{v.z, v.w}}, dfc_load(A + (j0 + lane) + (size_t)(j0 + q) * n),
                                    dfc{df{xq.x, xq.y}, df{xq.z, xq.w}});
                    v = make_float4(r.re.h, r.re.l, r.im.h, r.im.l);
                }
            }
            if (lane < jb) x[j0 + lane] = v;
        }
        __syncthreads();
        for (int i = tid; i < j0; i += NT) {
            dfc acc = dfc_load(x + i);
            for (int q = 0; q < jb; ++q) acc = dfc_fms(acc, dfc_load(A + i + (size_t)(j0 + q) * n), dfc_load(x + j0 + q));
            dfc_store(x + i, acc);
        }
        __syncthreads();
    }
}

// a = M^-1 phi by the mixed LU plus iterative refinement: r = phi - M a with
// M in FP64 for the refinement residual: every element evaluated as the FP64
// engine does (each pair on its own, so the writes stay coalesced)
static __device__ void assemble_fp64_copy(zc* __restrict__ M, const MedDev& md, zc k, MixSmem& s) {
    const int n = md.n;
    const zc dg = s.diag[0];
    for (size_t e = threadIdx.x; e < (size_t)n * n; e += NT) {
        const int i = (int)(e % n), j = (int)(e / n);
        zc m = dg, dm;
        if (i != j) pair_elements(md.d, k, atom_distance(md.d, md.pos, min(i, j), max(i, j)), false, m, dm);
        M[e] = m;
    }
    __syncthreads();
}

// a = M^-1 phi from the mixed LU with iterative refinement: r = phi - M a in
// FP64 against the FP64 copy of M, a += (LU)^-1 r (correction in double-float,
// a kept in FP64), until |r| <= 1e-14 |phi| (max norms), the residual stops
// halving, or 8 corrections.  Returns sigma = -Im(conj(phi).a)/k (the optical
// theorem of total_cross_section, ms_matrix_util.c:361).
static __device__ zc refine_solve(const float4* __restrict__ LU, const zc* __restrict__ M, const zc* __restrict__ phi,
                           zc* __restrict__ x, float4* __restrict__ r, float4* __restrict__ t, const MedDev& md,
                           zc k, const int* __restrict__ ipiv, MixSmem& s) {
    const int n = md.n, tid = threadIdx.x;
    auto to4 = [](zc v) {
        const df a = df_from_double(v.re), b = df_from_double(v.im);
        return make_float4(a.h, a.l, b.h, b.l);
    };
    for (int i = tid; i < n; i += NT) t[i] = to4(phi[i]);
    __syncthreads();
    df_solve_vec(LU, t, n, ipiv, s);
    for (int i = tid; i < n; i += NT) {
        const dfc v = dfc_load(t + i);
        x[i] = mk(df_to_double(v.re), df_to_double(v.im));
    }
    __syncthreads();
    double pmax = 0.0;
    for (int i = tid; i < n; i += NT) pmax = fmax(pmax, zabs(phi[i]));
    int dummy;
    block_argmax(pmax, tid, s, dummy);
    pmax = block_max_value(s);
    __syncthreads();
    double prev = INFINITY;
    for (int it = 0; it < 8; ++it) {
        // r = phi - M x in FP64, rows over threads (coalesced columns of M)
        double rmax = 0.0;
        for (int i = tid; i < n; i += NT) {
            zc acc = phi[i];
            for (int j = 0; j < n; ++j) {
                const zc mv = M[i + (size_t)j * n], xv = x[j];
                acc.re = fma(-mv.re, xv.re, fma(mv.im, xv.im, acc.re));
                acc.im = fma(-mv.re, xv.im, fma(-mv.im, xv.re, acc.im));
            }
            r[i] = to4(acc);
            rmax = fmax(rmax, fabs(acc.re) + fabs(acc.im));
        }
        block_argmax(rmax, tid, s, dummy);
        rmax = block_max_value(s);
        __syncthreads();
        if (!(rmax > 1e-14 * pmax) || !(rmax < 0.5 * prev)) break;
        prev = rmax;
        df_solve_vec(LU, r, n, ipiv, s);
        for (int i = tid; i < n; i += NT) {
            const dfc v = dfc_load(r + i);
            x[i] = x[i] + mk(df_to_double(v.re), df_to_double(v.im));
        }
        __syncthreads();
    }
    double dr = 0.0, di = 0.0, z = 0.0;
    for (int i = tid; i < n; i += NT) {
        const zc tt = conjz(phi[i]) * x[i];
        dr += tt.re;
        di += tt.im;
    }
    block_sum3(dr, di, z, s);
    return mk(-di, 0.0) / k;
}

// One instantiation per job kind (0 ln det, 1 dlogf, 2 amplitudes) and per
// dimension class (D3ONLY: every medium of the job has d = 3): each carries
// only its own reduction, solve and Green function, so a kernel's registers
// are not shaped by code it never runs (a never-taken call to the d != 3 tile
// cost the d = 3 ln det kernel 5 %).
// host entries of the six variants (mixed_k*.cu): set the shared-memory limit
// (attr_only) or launch
int mixed_variant_0_d3(const EngineParams&, const MixScratch&, int, size_t, cudaStream_t, bool);
int mixed_variant_1_d3(const EngineParams&, const MixScratch&, int, size_t, cudaStream_t, bool);
int mixed_variant_2_d3(const EngineParams&, const MixScratch&, int, size_t, cudaStream_t, bool);
int mixed_variant_0_any(const EngineParams&, const MixScratch&, int, size_t, cudaStream_t, bool);
int mixed_variant_1_any(const EngineParams&, const MixScratch&, int, size_t, cudaStream_t, bool);
int mixed_variant_2_any(const EngineParams&, const MixScratch&, int, size_t, cudaStream_t, bool);

#ifdef MSG_MIXED_KERNEL_BODY
template <int KIND, bool D3ONLY>
__global__ void __launch_bounds__(NT, 2) k_engine_mixed(EngineParams P, MixScratch X)
{
    extern __shared__ uint8_t smem_raw[];
    MixSmem& s = *reinterpret_cast<MixSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        tmem_alloc(&s.tmem, TMEM_COLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&s.bar_a, 1);
        mbar_init(&s.bar_b, 1);
        mbar_init(&s.bar_mma, 1);
        s.err = 0;
        s.mma_stuck = 0;
        for (int i = 0; i < PH_N; ++i) s.stat[i] = 0;
        fence_mbar_init();
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s.tmem;
    Phases ph{0, 0, 0};
    const size_t vec = (((size_t)P.piv_stride + 15) / 16) * 16;
    const size_t slot_all = KIND == 0 ? P.slot : (KIND == 1 ? 2 * P.slot : 2 * P.slot + 4 * vec);
    float4* A = reinterpret_cast<float4*>(P.ws) + (size_t)blockIdx.x * slot_all;
    float4* B = (KIND == 1) ? A + P.slot : nullptr;
    // kind 2: copy of M, right-hand side phi, solution, residual, correction
    zc* Mc = reinterpret_cast<zc*>(A + P.slot);  // kind 2: M in FP64 for the refinement
    zc* vphi = reinterpret_cast<zc*>(A + 2 * P.slot);
    zc* vx = vphi + vec;
    float4* vr = reinterpret_cast<float4*>(vx + vec);
    float4* vt = vr + vec;
    int* ipiv = P.piv + (size_t)blockIdx.x * P.piv_stride;
    bool alive = true;
    while (alive) {
        if (tid == 0) {
            const unsigned q = atomicAdd(P.counter, 1u);
            s.item = q < P.counter[1] ? (int)q : P.nitem;
            s.info = 0;
        }
        __syncthreads();
        const int q = s.item;
        if (q >= P.nitem) break;
        const int it = P.order[q];
        const MedDev md = P.media[P.item_med[it]];
        const zc k = mk(P.ks[2 * it], P.ks[2 * it + 1]);
        stat_start(s);
        const float2 rg = assemble_df<D3ONLY>(A, B, md.n, md.d, md.pos, md.model, k, s);
        stat_add(s, PH_ASSEMBLE);
        int dummy;
        block_argmax((double)rg.x, tid, s, dummy);
        const double mxd = block_max_value(s);
        __syncthreads();  // red_v is reused by the next reduction
        block_argmax(-(double)rg.y, tid, s, dummy);
        const double mnd = -block_max_value(s);
        __syncthreads();
        // six slices when the entries span more than SPAN_WIDE (SPAN_WIDE_REFINED for amplitude
        // items) or an entry is zero / non-finite, and for every dlogf item (near a root the condition number of M magnifies the LU's
        // error in tr(M^-1 dM/dk)), if this launch has the shared memory for them; else four,
        // and a status bit says so
        const double thr = KIND == 2 ? (double)SPAN_WIDE_REFINED : (double)SPAN_WIDE;
        const bool span_wide = KIND == 1 || !(mxd <= thr * mnd);
        const bool wide = span_wide && P.wide_ok;
        zc res = mk(0.0);
        int st = 0;
        if (!(mxd < (double)RANGE_LIMIT)) {
            st |= MSGPU_S_RANGE;
            res = mk(nan(""), nan(""));
        } else {
            if (KIND == 2) {
                // keep M for the residual; incident plane wave along +x (incident_wave_util.c:76)
                assemble_fp64_copy(Mc, md, k, s);
                for (int i = tid; i < md.n; i += NT) vphi[i] = zexp(mk(0.0, 1.0) * k * md.pos[i * md.d]);
                __syncthreads();
            }
            if (!(wide ? lu_mixed<6>(A, md.n, ipiv, KIND != 0, s, X, tmem, ph)
                       : lu_mixed<4>(A, md.n, ipiv, KIND != 0, s, X, tmem, ph))) {
                alive = false;
            } else if (KIND == 0) {
                res = tracelog_df(A, md.n, ipiv, s);
            } else if (KIND == 1) {
                if (!(wide ? trace_solve_mixed<6>(A, B, md.n, ipiv, s, X, tmem, ph, res)
                           : trace_solve_mixed<4>(A, B, md.n, ipiv, s, X, tmem, ph, res)))
                    alive = false;
            } else {
                res = refine_solve(A, Mc, vphi, vx, vr, vt, md, k, ipiv, s);
                if (P.amps)
                    for (int i = tid; i < md.n; i += NT) {
                        P.amps[2 * (P.amp_off[it] + i)] = vx[i].re;
                        P.amps[2 * (P.amp_off[it] + i) + 1] = vx[i].im;
                    }
            }
        }
        if (!alive) {
            st |= MSGPU_S_TIMEOUT;
            res = mk(nan(""), nan(""));
        }
        if (tid == 0) {
            s.stat[PH_ITEMS] += 1;
            if (span_wide && !wide) st |= MSGPU_S_SPAN;
            P.out[2 * it] = res.re;
            P.out[2 * it + 1] = res.im;
            if (s.info) st |= MSGPU_S_SINGULAR;
            if (!isfinite(res.re) || !isfinite(res.im)) st |= MSGPU_S_NONFINITE;
            P.status[it] = st;
        }
        __syncthreads();
    }
    if (s.err && tid == 0) {
        atomicExch(X.err, 1);
        // the run is abandoned: every item not yet taken is marked, none keeps a stale result
        for (unsigned q = atomicAdd(P.counter, 1u); q < P.counter[1] && (int)q < P.nitem;
             q = atomicAdd(P.counter, 1u)) {
            const int it = P.order[q];
            P.out[2 * it] = P.out[2 * it + 1] = nan("");
            P.status[it] = MSGPU_S_TIMEOUT;
        }
    }
    if (X.stats && tid == 0)
        for (int i = 0; i < PH_N; ++i) atomicAdd(X.stats + i, s.stat[i]);
    // an MMA completion wait that ran out may leave MMAs in flight: give them a bounded chance to land
    if (s.mma_stuck && tid == 0) mbar_wait(&s.bar_mma, (uint32_t)(s.mma_stuck - 1), 1 << 20);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TMEM_COLS);
}
#endif

}  // namespace msg
