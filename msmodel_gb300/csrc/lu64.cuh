// lu64.cuh -- CTA-level FP64 complex dense kernels: blocked right-looking
// LU with partial pivoting, the triangular solves of LAPACK zgetrs, and the
// Foldy-Lax matrix assembly.  One CTA owns one matrix in global memory
// (column-major, leading dimension n) and works on it alone, so thousands of
// (k, realisation) matrices factor concurrently with no inter-CTA traffic.
//
// The FP64 pipe of GB300 is the roofline of this path (about 2 FP64 FMA
// lanes per SM per clock): every loop below keeps the SM's FP64 FMAs fed
// from shared-memory tiles; memory traffic is a few percent of the time.
//
// Pivoting follows LAPACK zgetf2/zgetrf: the pivot of column j is the first
// row of maximum |Re|+|Im| (IZAMAX), ipiv is kept 0-based here, interchanges
// are applied to whole rows (LAPACK layout of L), a zero pivot sets info and
// skips the scaling, the multipliers are scaled by the reciprocal of the
// pivot when |pivot| >= DBL_MIN and divided otherwise.
#pragma once
#include <float.h>
#include "cplx.cuh"
#include "green.cuh"

namespace msg {

constexpr int NT = 256;  // threads per CTA
constexpr int NB = 32;   // panel width
constexpr int TM = 64;   // trailing-update tile rows
constexpr int TN = 64;   // trailing-update tile columns

struct __align__(16) LuSmem {
    zc As[NB][TM];       // 32 KB  L21 tile  (k-major)
    zc Bs[NB][TN];       // 32 KB  U12 tile  (k-major)
    zc T[NB][NB + 1];    // 16.5 KB diagonal block / assembly transpose
    zc urow[NB];         // pivot row of the panel
    zc diag[2];          // F^-1(k), d F^-1/dk
    double red_v[NT / 32];
    int red_i[NT / 32];
    double red_s[3][NT / 32];
    int info;
    int bcast_i;
    int item;
};

template <class S>
__device__ __forceinline__ void block_argmax(double v, int i, S& s, int& oi) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        double v2 = __shfl_down_sync(FULL, v, off);
        int i2 = __shfl_down_sync(FULL, i, off);
        if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
    }
    if (lane == 0) { s.red_v[warp] = v; s.red_i[warp] = i; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bv = s.red_v[0];
        int bi = s.red_i[0];
        for (int w = 1; w < NT / 32; w++) {
            double v2 = s.red_v[w];
            int i2 = s.red_i[w];
            if (v2 > bv || (v2 == bv && i2 < bi)) { bv = v2; bi = i2; }
        }
        s.bcast_i = bi;
    }
    __syncthreads();
    oi = s.bcast_i;
}

// sum of three doubles over the CTA; result valid in every thread
template <class S>
__device__ __forceinline__ void block_sum3(double& a, double& b, double& c, S& s) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(FULL, a, off);
        b += __shfl_down_sync(FULL, b, off);
        c += __shfl_down_sync(FULL, c, off);
    }
    if (lane == 0) { s.red_s[0][warp] = a; s.red_s[1][warp] = b; s.red_s[2][warp] = c; }
    __syncthreads();
    a = b = c = 0.0;
    for (int w = 0; w < NT / 32; w++) { a += s.red_s[0][w]; b += s.red_s[1][w]; c += s.red_s[2][w]; }
    __syncthreads();
}

// Factor the panel A[j0:n, j0:j0+jb) in place; interchanges inside the panel only.
static __device__ void panel_factor(zc* __restrict__ A, int n, int j0, int jb, int* __restrict__ ipiv, LuSmem& s) {
    const int tid = threadIdx.x;
    const int cend = j0 + jb;
    double bv = -1.0;
    int bi = n;
    for (int i = j0 + tid; i < n; i += NT) {
        double v = abs1(A[i + (size_t)j0 * n]);
        if (v > bv) { bv = v; bi = i; }
    }
    for (int c = j0; c < cend; ++c) {
        int p;
        block_argmax(bv, bi, s, p);
        if (p >= n) p = c;
        const zc piv = A[p + (size_t)c * n];
        const bool nz = !is_zero(piv);
        if (tid == 0) {
            ipiv[c] = p;
            if (!nz && s.info == 0) s.info = c + 1;
        }
        __syncthreads();  // every thread holds the pivot before row p is swapped away
        if (nz && p != c && tid < jb) {
            const size_t col = (size_t)(j0 + tid) * n;
            zc t = A[c + col];
            A[c + col] = A[p + col];
            A[p + col] = t;
        }
        __syncthreads();
        if (tid < jb && j0 + tid > c) s.urow[tid] = A[c + (size_t)(j0 + tid) * n];
        __syncthreads();
        bv = -1.0;
        bi = n;
        if (nz) {
            const bool recip = zabs(piv) >= DBL_MIN;
            const zc r = recip ? 1.0 / piv : mk(0.0);
            for (int i = c + 1 + tid; i < n; i += NT) {
                zc l = A[i + (size_t)c * n];
                l = recip ? l * r : l / piv;
                A[i + (size_t)c * n] = l;
                if (c + 1 < cend) {
                    zc a = A[i + (size_t)(c + 1) * n] - l * s.urow[c + 1 - j0];
                    A[i + (size_t)(c + 1) * n] = a;
                    double v = abs1(a);
                    if (v > bv) { bv = v; bi = i; }
                    for (int cc = c + 2; cc < cend; ++cc) {
                        zc* q = A + i + (size_t)cc * n;
                        *q = *q - l * s.urow[cc - j0];
                    }
                }
            }
        } else if (c + 1 < cend) {
            for (int i = c + 1 + tid; i < n; i += NT) {
                double v = abs1(A[i + (size_t)(c + 1) * n]);
                if (v > bv) { bv = v; bi = i; }
            }
        }
    }
    __syncthreads();
}

// Column solves used by the blocked TRSM steps.  One thread owns one column
// b[0..jb) (global memory); the jb x jb triangle sits in s.T.  Rows are
// processed in chunks of CH so that only CH complex values live in registers;
// solved values of earlier chunks are re-read from memory.
constexpr int CH = 8;

__device__ __forceinline__ void col_solve_lower_unit(zc* __restrict__ b, int jb, const zc (*T)[NB + 1]) {
    for (int rb = 0; rb < jb; rb += CH) {
        zc y[CH];
#pragma unroll
        for (int r = 0; r < CH; ++r) y[r] = (rb + r < jb) ? b[rb + r] : mk(0.0);
        for (int q = 0; q < rb; ++q) {
            const zc xq = b[q];
#pragma unroll
            for (int r = 0; r < CH; ++r) y[r] -= T[rb + r][q] * xq;
        }
#pragma unroll
        for (int r = 1; r < CH; ++r)
#pragma unroll
            for (int q = 0; q < r; ++q) y[r] -= T[rb + r][rb + q] * y[q];
#pragma unroll
        for (int r = 0; r < CH; ++r)
            if (rb + r < jb) b[rb + r] = y[r];
    }
}

__device__ __forceinline__ void col_solve_upper(zc* __restrict__ b, int jb, const zc (*T)[NB + 1]) {
    for (int rb = ((jb - 1) / CH) * CH; rb >= 0; rb -= CH) {
        zc y[CH];
#pragma unroll
        for (int r = 0; r < CH; ++r) y[r] = (rb + r < jb) ? b[rb + r] : mk(0.0);
        for (int q = rb + CH; q < jb; ++q) {
            const zc xq = b[q];
#pragma unroll
            for (int r = 0; r < CH; ++r) y[r] -= T[rb + r][q] * xq;
        }
#pragma unroll
        for (int r = CH - 1; r >= 0; --r) {
            if (rb + r < jb) {
                zc acc = y[r];
#pragma unroll
                for (int q = r + 1; q < CH; ++q) acc -= T[rb + r][rb + q] * y[q];
                y[r] = acc / T[rb + r][rb + r];
            }
        }
#pragma unroll
        for (int r = 0; r < CH; ++r)
            if (rb + r < jb) b[rb + r] = y[r];
    }
}

// Apply the panel's interchanges to every other column and compute
// U12 = L11^-1 A12 (columns right of the panel).
static __device__ void panel_swaps_trsm(zc* __restrict__ A, int n, int j0, int jb, const int* __restrict__ ipiv,
                                 LuSmem& s) {
    const int tid = threadIdx.x;
    for (int e = tid; e < NB * NB; e += NT) {
        int r = e % NB, q = e / NB;
        s.T[r][q] = (r < jb && q < r) ? A[(j0 + r) + (size_t)(j0 + q) * n] : mk(0.0);
    }
    __syncthreads();
    for (int col = tid; col < n; col += NT) {
        if (col >= j0 && col < j0 + jb) continue;
        zc* a = A + (size_t)col * n;
        for (int c = j0; c < j0 + jb; ++c) {
            int p = ipiv[c];
            if (p != c) { zc t = a[c]; a[c] = a[p]; a[p] = t; }
        }
        if (col >= j0 + jb) col_solve_lower_unit(a + j0, jb, s.T);
    }
    __syncthreads();
}

// C[m x nn] -= Ablk[m x kk] * Bblk[kk x nn] (all column-major); kk <= NB.
// tri != 0: only tiles that hold some element with row >= col are updated
// (row/col counted from the C origin plus rofs/cofs).
static __device__ void gemm_sub(zc* __restrict__ C, int ldc, const zc* __restrict__ Ab, int lda, const zc* __restrict__ Bb,
                         int ldb, int m, int nn, int kk, LuSmem& s, int tri = 0, int rofs = 0, int cofs = 0) {
    if (m <= 0 || nn <= 0 || kk <= 0) return;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    for (int ti = 0; ti < m; ti += TM) {
        if (tri && rofs + ti + TM - 1 < cofs) continue;  // whole row band above every column
        for (int e = tid; e < NB * TM; e += NT) {
            int r = e % TM, k = e / TM;
            zc v = mk(0.0);
            if (k < kk && ti + r < m) v = Ab[(ti + r) + (size_t)k * lda];
            s.As[k][r] = v;
        }
        for (int tj = 0; tj < nn; tj += TN) {
            if (tri && rofs + ti + TM - 1 < cofs + tj) break;
            for (int e = tid; e < NB * TN; e += NT) {
                int k = e % NB, c = e / NB;
                zc v = mk(0.0);
                if (k < kk && tj + c < nn) v = Bb[k + (size_t)(tj + c) * ldb];
                s.Bs[k][c] = v;
            }
            __syncthreads();
            zc acc[4][4];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    int r = ti + tx + 16 * a, c = tj + ty + 16 * b;
                    acc[a][b] = (r < m && c < nn) ? C[r + (size_t)c * ldc] : mk(0.0);
                }
#pragma unroll 2
            for (int k = 0; k < kk; ++k) {
                zc av[4], bw[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) av[a] = s.As[k][tx + 16 * a];
#pragma unroll
                for (int b = 0; b < 4; ++b) bw[b] = s.Bs[k][ty + 16 * b];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        acc[a][b].re = fma(-av[a].re, bw[b].re, acc[a][b].re);
                        acc[a][b].re = fma(av[a].im, bw[b].im, acc[a][b].re);
                        acc[a][b].im = fma(-av[a].re, bw[b].im, acc[a][b].im);
                        acc[a][b].im = fma(-av[a].im, bw[b].re, acc[a][b].im);
                    }
            }
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    int r = ti + tx + 16 * a, c = tj + ty + 16 * b;
                    if (r < m && c < nn) C[r + (size_t)c * ldc] = acc[a][b];
                }
            __syncthreads();
        }
    }
}

// In-place LU of A (n x n, ld n).  ipiv 0-based.  Sets s.info (1-based first zero pivot).
static __device__ void lu_factor(zc* __restrict__ A, int n, int* __restrict__ ipiv, LuSmem& s) {
    for (int j0 = 0; j0 < n; j0 += NB) {
        const int jb = min(NB, n - j0);
        panel_factor(A, n, j0, jb, ipiv, s);
        panel_swaps_trsm(A, n, j0, jb, ipiv, s);
        const int r0 = j0 + jb;
        gemm_sub(A + r0 + (size_t)r0 * n, n, A + r0 + (size_t)j0 * n, n, A + j0 + (size_t)r0 * n, n, n - r0, n - r0,
                 jb, s);
    }
}

// ln det(A)/n with the reference's branch: sum log|U_ii| + i (sum Arg U_ii + pi [odd interchanges]).
static __device__ zc lu_tracelog(const zc* __restrict__ A, int n, const int* __restrict__ ipiv, LuSmem& s) {
    double lr = 0.0, ar = 0.0, odd = 0.0;
    for (int i = threadIdx.x; i < n; i += NT) {
        zc u = A[i + (size_t)i * n];
        lr += log(hypot(u.re, u.im));
        ar += atan2(u.im, u.re);
        if (ipiv[i] != i) odd += 1.0;
    }
    block_sum3(lr, ar, odd, s);
    if (fmod(odd, 2.0) == 1.0) ar += PI;
    return mk(lr / n, ar / n);
}

// tr(A^-1 B) given the LU of A (LAPACK layout) and B (n x n, ld n), B destroyed:
// B <- P B, forward solve with unit-lower L, backward solve with U restricted
// to the rows each diagonal element needs (X_jj depends on rows >= j only).
static __device__ zc lu_trace_solve(const zc* __restrict__ A, zc* __restrict__ B, int n, const int* __restrict__ ipiv,
                             LuSmem& s) {
    const int tid = threadIdx.x;
    for (int col = tid; col < n; col += NT) {
        zc* b = B + (size_t)col * n;
        for (int i = 0; i < n; ++i) {
            int p = ipiv[i];
            if (p != i) { zc t = b[i]; b[i] = b[p]; b[p] = t; }
        }
    }
    __syncthreads();
    // forward: L X = P B
    for (int j0 = 0; j0 < n; j0 += NB) {
        const int jb = min(NB, n - j0);
        for (int e = tid; e < NB * NB; e += NT) {
            int r = e % NB, q = e / NB;
            s.T[r][q] = (r < jb && q < r) ? A[(j0 + r) + (size_t)(j0 + q) * n] : mk(0.0);
        }
        __syncthreads();
        for (int col = tid; col < n; col += NT) col_solve_lower_unit(B + (size_t)col * n + j0, jb, s.T);
        __syncthreads();
        const int r0 = j0 + jb;
        gemm_sub(B + r0, n, A + r0 + (size_t)j0 * n, n, B + j0, n, n - r0, n, jb, s);
    }
    // backward: U X = Y, columns [0, j0+jb) of block row j0 only
    const int nblk = (n + NB - 1) / NB;
    for (int kb = nblk - 1; kb >= 0; --kb) {
        const int j0 = kb * NB, jb = min(NB, n - j0), ncol = j0 + jb;
        for (int e = tid; e < NB * NB; e += NT) {
            int r = e % NB, q = e / NB;
            s.T[r][q] = (r < jb && q < jb && q >= r) ? A[(j0 + r) + (size_t)(j0 + q) * n] : mk(r == q ? 1.0 : 0.0);
        }
        __syncthreads();
        for (int col = tid; col < ncol; col += NT) col_solve_upper(B + (size_t)col * n + j0, jb, s.T);
        __syncthreads();
        // Y[0:j0, 0:ncol] -= U[0:j0, j0:j0+jb] X[j0:j0+jb, 0:ncol]   (rows >= cols only)
        gemm_sub(B, n, A + (size_t)j0 * n, n, B + j0, n, j0, ncol, jb, s, 1, 0, 0);
    }
    double tr = 0.0, ti = 0.0, z = 0.0;
    for (int i = tid; i < n; i += NT) {
        zc v = B[i + (size_t)i * n];
        tr += v.re;
        ti += v.im;
    }
    block_sum3(tr, ti, z, s);
    return mk(tr, ti);
}

// x <- A^-1 x for one right-hand side x[n] (global), LAPACK-layout LU: the
// interchanges, then blocked forward and backward substitution; each block's
// small triangle is solved by warp 0 (one row per lane), the rectangular
// remainder by all threads (one row per thread, coalesced column reads).
static __device__ void lu_solve_vec(const zc* __restrict__ A, zc* __restrict__ x, int n, const int* __restrict__ ipiv,
                             LuSmem& s) {
    const unsigned FULL = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid == 0)
        for (int i = 0; i < n; ++i) {
            int p = ipiv[i];
            if (p != i) { zc t = x[i]; x[i] = x[p]; x[p] = t; }
        }
    __syncthreads();
    for (int j0 = 0; j0 < n; j0 += NB) {
        const int jb = min(NB, n - j0);
        if (tid < 32) {
            zc v = lane < jb ? x[j0 + lane] : mk(0.0);
            for (int q = 0; q < jb - 1; ++q) {
                zc xq = mk(__shfl_sync(FULL, v.re, q), __shfl_sync(FULL, v.im, q));
                if (lane > q && lane < jb) v -= A[(j0 + lane) + (size_t)(j0 + q) * n] * xq;
            }
            if (lane < jb) x[j0 + lane] = v;
        }
        __syncthreads();
        for (int i = j0 + jb + tid; i < n; i += NT) {
            zc acc = x[i];
            for (int q = 0; q < jb; ++q) acc -= A[i + (size_t)(j0 + q) * n] * x[j0 + q];
            x[i] = acc;
        }
        __syncthreads();
    }
    const int nblk = (n + NB - 1) / NB;
    for (int kb = nblk - 1; kb >= 0; --kb) {
        const int j0 = kb * NB, jb = min(NB, n - j0);
        if (tid < 32) {
            zc v = lane < jb ? x[j0 + lane] : mk(0.0);
            for (int q = jb - 1; q >= 0; --q) {
                if (lane == q) v = v / A[(j0 + q) + (size_t)(j0 + q) * n];
                zc xq = mk(__shfl_sync(FULL, v.re, q), __shfl_sync(FULL, v.im, q));
                if (lane < q) v -= A[(j0 + lane) + (size_t)(j0 + q) * n] * xq;
            }
            if (lane < jb) x[j0 + lane] = v;
        }
        __syncthreads();
        for (int i = tid; i < j0; i += NT) {
            zc acc = x[i];
            for (int q = 0; q < jb; ++q) acc -= A[i + (size_t)(j0 + q) * n] * x[j0 + q];
            x[i] = acc;
        }
        __syncthreads();
    }
}

// Off-diagonal matrix elements -G (and -dG/dk) for one pair distance.
__device__ __forceinline__ void pair_elements(int d, zc k, double r, bool want_deriv, zc& m, zc& dm) {
    if (d == 3) {
        // G = -e^{ikr}/(4 pi r);  dG/dk = (k/2pi) G_1 = (k/2pi) e^{ikr}/(2ik) = -i e^{ikr}/(4pi)
        zc e = zexp(mk(-k.im * r, k.re * r));
        m = e / (FOURPI * r);
        if (want_deriv) dm = mk(-e.im, e.re) / FOURPI;
        return;
    }
    m = -free_green(d, k, r);
    if (want_deriv) dm = -dk_free_green(d, k, r);
}

// K_nu regime of the pair's argument z = -i k r (the reference's switch,
// green_bessel.c:208-218): 0 asymptotic, 1 ascending series, 2 Miller.
__device__ __forceinline__ int k_regime(zc k, double r) {
    const double x = k.im * r, y = -k.re * r;
    if (x * x + y * y > 256.0) return 0;
    if (x < 3.0 - y * y / 12.0) return 1;
    return 2;
}

// Pairs i < j of the 32 x 32 tile (I, J) for d != 3, evaluated grouped by K_nu
// regime: the three loops differ several-fold in length, and a warp that
// mixes them runs all of them.  Every pair goes to one of three lists in
// shared memory (list: 3 x 1024 entries, cnt: 3 counters, both zero on entry
// and on return), then consecutive threads take consecutive list entries;
// put(ii, jj, m, dm) receives each element.  Entries of a list are in no
// fixed order, but every element is a function of (k, r) alone.
template <class Put>
__device__ __forceinline__ void tile_pairs_grouped(int I, int J, int n, int d, const double* __restrict__ pos, zc k,
                                                   bool want_deriv, unsigned short* list, int* cnt, Put put) {
    const int tid = threadIdx.x;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int p = tid + NT * q, ii = p & 31, jj = p >> 5;
        const int i = I * 32 + ii, j = J * 32 + jj;
        if (i < n && j < n && i < j) {
            const int reg = k_regime(k, atom_distance(d, pos, i, j));
            list[reg * 1024 + atomicAdd(&cnt[reg], 1)] = (unsigned short)p;
        }
    }
    __syncthreads();
    const int c0 = cnt[0], c1 = cnt[1], tot = c0 + c1 + cnt[2];
    for (int w = tid; w < tot; w += NT) {
        const int p = w < c0 ? list[w] : (w < c0 + c1 ? list[1024 + w - c0] : list[2048 + w - c0 - c1]);
        const int ii = p & 31, jj = p >> 5;
        zc m, dm = mk(0.0);
        pair_elements(d, k, atom_distance(d, pos, I * 32 + ii, J * 32 + jj), want_deriv, m, dm);
        put(ii, jj, m, dm);
    }
    __syncthreads();
    if (tid < 3) cnt[tid] = 0;
}

// Assemble M(k) into A and, if B != nullptr, dM/dk into B (ld n, column-major).
// Tiles of 32 x 32 pairs above the diagonal are evaluated once and written to
// both triangles, the mirrored tile through shared memory to keep stores coalesced.
static __device__ void assemble(zc* __restrict__ A, zc* __restrict__ B, int n, int d, const double* __restrict__ pos,
                         const msgpu_model& mdl, zc k, LuSmem& s) {
    const int tid = threadIdx.x;
    if (tid == 0) {
        s.diag[0] = invf(mdl, d, k);
        if (B) s.diag[1] = dk_invf(mdl, d, k);
    }
    __syncthreads();
    const zc dg0 = s.diag[0], dg1 = s.diag[1];
    zc (*T2)[NB + 1] = reinterpret_cast<zc(*)[NB + 1]>(&s.As[0][0]);
    // d != 3: pair lists of the regime grouping in the (idle) U12 tile buffer
    unsigned short* list = reinterpret_cast<unsigned short*>(&s.Bs[0][0]);
    int* cnt = reinterpret_cast<int*>(list + 3 * 1024);
    const bool grouped = d != 3 && d != 1;
    if (grouped && tid < 3) cnt[tid] = 0;
    __syncthreads();
    const int nt = (n + 31) / 32;
    for (int J = 0; J < nt; ++J) {
        for (int I = 0; I <= J; ++I) {
            if (grouped) {
                tile_pairs_grouped(I, J, n, d, pos, k, B != nullptr, list, cnt, [&](int ii, int jj, zc m, zc dm) {
                    s.T[jj][ii] = m;
                    if (B) T2[jj][ii] = dm;
                });
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int ii = tid & 31, jj = (tid >> 5) + 8 * q;
                    const int i = I * 32 + ii, j = J * 32 + jj;
                    if (i < n && j < n && i <= j) {
                        A[i + (size_t)j * n] = i < j ? s.T[jj][ii] : dg0;
                        if (B) B[i + (size_t)j * n] = i < j ? T2[jj][ii] : dg1;
                    }
                }
            } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int ii = tid & 31, jj = (tid >> 5) + 8 * q;
                const int i = I * 32 + ii, j = J * 32 + jj;
                if (i < n && j < n && i <= j) {
                    zc m, dm = mk(0.0);
                    if (i < j) {
                        pair_elements(d, k, atom_distance(d, pos, i, j), B != nullptr, m, dm);
                    } else {
                        m = dg0;
                        dm = dg1;
                    }
                    A[i + (size_t)j * n] = m;
                    s.T[jj][ii] = m;
                    if (B) {
                        B[i + (size_t)j * n] = dm;
                        T2[jj][ii] = dm;
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
                    A[j + (size_t)i * n] = s.T[jj][ii];
                    if (B) B[j + (size_t)i * n] = T2[jj][ii];
                }
            }
            __syncthreads();
        }
    }
}

}  // namespace msg
