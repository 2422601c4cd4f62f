// eigvals.cu -- the eigenvalues mu of M(k), the input of the reference's
// mu-plane histograms (eigvals, src/core/ms_matrix_util.c:147, zgeev_ without
// eigenvectors; run_chistogram_omp and run_imag_mu_histogram_omp,
// src/core/ms_core.c:173-282).
//
// One persistent CTA per matrix slot, FP64 throughout (the reference's
// arithmetic), items dealt to CTAs in order:
//   1. M(k) assembled by the FP64 engine's assembly (lu64.cuh), or the
//      normalized N(k) = i - G(k)/I(k,0) of the mu-plane task's mtype=normalized
//      (build_normalized_matrix, ms_matrix_util.c:50) made from it in place;
//   2. reduction to upper Hessenberg form by Householder reflectors, as
//      LAPACK's unblocked zgehd2 (reflector of zlarfg; H applied from the
//      right to rows 0..n-1, H^H from the left to the trailing rows), the
//      reflector in shared memory, the right update one thread per row and the
//      left update one warp per column (coalesced both ways);
//   3. eigenvalues of the Hessenberg matrix by the single-shift complex QR
//      algorithm of LAPACK's zlahqr with wantt = wantz = false (real
//      subdiagonals, the Ahues-Kressner deflation test, Wilkinson shifts with
//      exceptional shifts every 10 iterations without deflation, the search
//      for two consecutive small subdiagonals, 2 x 2 reflectors chasing the
//      bulge through the active block): thread 0 takes the scalar chain of
//      each bulge step, the CTA splits the step's row and column updates.
// zgeev also balances the matrix first (zgebal); this path does not: M(k)'s
// entries do not span the magnitudes balancing is for, and the eigenvalues
// agree with the reference's to ~1e-13 of the largest.  Eigenvalues come out
// in deflation order, as zgeev's.
#include <cuda_runtime.h>
#include <float.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include "msgpu.h"
#include "lu64.cuh"
#include "engine_internal.h"

namespace msg {

// shared memory: the assembly's and the reductions' LuSmem; the Householder
// vector overlays its two tile buffers (4096 complex values: n <= 4097)
constexpr int EIG_NMAX = NB * (TM + TN) + 1;

struct EigParams {
    int nitem;
    const int* item_n;       // order per item
    const int* item_d;
    const size_t* item_pos;  // offset of the item's positions in pos
    const msgpu_model* item_model;
    const double* pos;
    const double* ks;        // 2 per item
    const size_t* item_out;  // offset of the item's eigenvalues in mu
    zc* mu;
    int* status;
    zc* work;                // one nmax x nmax slot per CTA
    size_t slot;
    int normalized;          // N(k) = i - G(k)/I(k,0) in place of M(k)
    double* trg2;            // per item Tr[G^+ G]/N of the matrix (tracegtwo), or nullptr
};

__device__ __forceinline__ double dlapy3(double x, double y, double z) {
    const double w = fmax(fabs(x), fmax(fabs(y), fabs(z)));
    if (w == 0.0) return fabs(x) + fabs(y) + fabs(z);
    const double a = x / w, b = y / w, c = z / w;
    return w * sqrt(a * a + b * b + c * c);
}

// Householder reduction to upper Hessenberg form (zgehd2, ilo = 1, ihi = n)
static __device__ void hessenberg(zc* __restrict__ A, int n, LuSmem& s) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    zc* v = &s.As[0][0];
    for (int j = 0; j + 2 < n; ++j) {
        const int m = n - j - 1;  // length of the reflector
        zc* col = A + (size_t)j * n + j + 1;
        double ss = 0.0, z1 = 0.0, z2 = 0.0;
        for (int i = 1 + tid; i < m; i += NT) ss += zabs2(col[i]);
        block_sum3(ss, z1, z2, s);
        const zc alpha = col[0];
        __syncthreads();  // every thread has read alpha before column j changes
        if (ss == 0.0 && alpha.im == 0.0) continue;  // H = I (tau = 0)
        // zlarfg: beta = -sign(Re alpha) |(alpha, x)|, tau = (beta - alpha) / beta,
        // v = (1, x / (alpha - beta))
        const double beta = -copysign(dlapy3(alpha.re, alpha.im, sqrt(ss)), alpha.re);
        const zc tau = mk((beta - alpha.re) / beta, -alpha.im / beta);
        const zc scal = 1.0 / (alpha - beta);
        for (int i = tid; i < m; i += NT) {
            v[i] = i == 0 ? mk(1.0) : col[i] * scal;
            col[i] = i == 0 ? mk(beta) : mk(0.0);
        }
        __syncthreads();
        // from the right: A[0:n, j+1:n] -= tau (A v) v^H
        for (int r = tid; r < n; r += NT) {
            zc* row = A + r + (size_t)(j + 1) * n;
            zc w = mk(0.0);
            for (int c = 0; c < m; ++c) w += row[(size_t)c * n] * v[c];
            w = tau * w;
            for (int c = 0; c < m; ++c) row[(size_t)c * n] -= w * conjz(v[c]);
        }
        __syncthreads();
        // from the left with conj(tau): A[j+1:n, j+1:n] -= conj(tau) v (v^H A)
        const zc ctau = conjz(tau);
        for (int c = j + 1 + warp; c < n; c += NT / 32) {
            zc* cc = A + (size_t)c * n + j + 1;
            zc w = mk(0.0);
            for (int i = lane; i < m; i += 32) w += conjz(v[i]) * cc[i];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                w.re += __shfl_xor_sync(0xffffffffu, w.re, off);
                w.im += __shfl_xor_sync(0xffffffffu, w.im, off);
            }
            w = ctau * w;
            for (int i = lane; i < m; i += 32) cc[i] -= v[i] * w;
        }
        __syncthreads();
    }
}

// zlarfg for n = 2: on return a = beta (real), x scaled, the reflector
// I - tau (1, x)(1, x)^H.  On the bulge-chasing chain of every QR step, so it
// takes two divisions and one square root (zlarfg's dlapy3 scaling guards
// against overflow of |a|^2 + |x|^2, far beyond M(k)'s entries)
__device__ __forceinline__ zc larfg2(zc& a, zc& x) {
    const double x2 = zabs2(x);
    if (x2 == 0.0 && a.im == 0.0) return mk(0.0);
    const double beta = -copysign(sqrt(a.re * a.re + a.im * a.im + x2), a.re);
    const double rb = 1.0 / beta;
    const zc tau = mk((beta - a.re) * rb, -a.im * rb);
    x = x * zrecip(a - beta);
    a = mk(beta);
    return tau;
}

// the QR iteration's scalars, computed by thread 0 and read by the CTA
struct HqrShared {
    zc t1, v2, temp;
    double t2;
    int l, m, flag;
};

// Eigenvalues of the upper Hessenberg H (n x n, ld n) into w by zlahqr's
// single-shift QR (wantt = wantz = false).  Thread 0 takes every scalar step
// (the deflation and shift searches, each 2 x 2 reflector) and the CTA splits
// each step's row and column updates, three barriers a bulge step.  (Letting
// thread 0 update the next reflector's two rows itself and start on it while
// the CTA finishes the step saves a barrier but measured 10-16% slower.)  Returns 0,
// or i + 1 if eigenvalue i and above did not converge within 30 max(10, n)
// iterations (zlahqr's info).
static __device__ int hqr_cta(zc* __restrict__ H, int n, zc* __restrict__ w, HqrShared& q) {
    const int tid = threadIdx.x;
    auto h = [&](int r, int c) -> zc& { return H[r + (size_t)c * n]; };
    if (n == 1) {
        if (tid == 0) w[0] = h(0, 0);
        return 0;
    }
    const int ilo = 0, ihi = n - 1;
    // subdiagonal entries made real by diagonal unitary similarity
    for (int i = ilo + 1; i <= ihi; ++i) {
        if (tid == 0) {
            const zc hs = h(i, i - 1);
            q.flag = hs.im != 0.0;
            if (q.flag) {
                const zc sc = hs / abs1(hs);
                q.temp = conjz(sc) / zabs(sc);
                h(i, i - 1) = mk(zabs(hs));
            }
        }
        __syncthreads();
        if (q.flag) {
            const zc sc = q.temp;
            for (int j = i + tid; j <= ihi; j += NT) h(i, j) = h(i, j) * sc;
            __syncthreads();
            const int top = min(ihi, i + 1);
            for (int j = ilo + tid; j <= top; j += NT) h(j, i) = h(j, i) * conjz(sc);
        }
        __syncthreads();
    }
    const double safmin = DBL_MIN, ulp = DBL_EPSILON;
    const double smlnum = safmin * ((double)(ihi - ilo + 1) / ulp);
    const int itmax = 30 * max(10, ihi - ilo + 1);
    constexpr int KEXSH = 10;
    int kdefl = 0;
    int i = ihi;
    zc v0 = mk(0.0), v1 = mk(0.0);  // thread 0's reflector vector
    while (i >= ilo) {
        int l = ilo;
        bool done = false;
        for (int its = 0; its <= itmax; ++its) {
            if (tid == 0) {
                // a single small subdiagonal element
                int k;
                for (k = i; k > l; --k) {
                    const zc hkk1 = h(k, k - 1);
                    if (abs1(hkk1) <= smlnum) break;
                    double tst = abs1(h(k - 1, k - 1)) + abs1(h(k, k));
                    if (tst == 0.0) {
                        if (k - 2 >= ilo) tst += fabs(h(k - 1, k - 2).re);
                        if (k + 1 <= ihi) tst += fabs(h(k + 1, k).re);
                    }
                    if (fabs(hkk1.re) <= ulp * tst) {
                        const double a1 = abs1(hkk1), a2 = abs1(h(k - 1, k));
                        const double ab = fmax(a1, a2), ba = fmin(a1, a2);
                        const double b1 = abs1(h(k, k)), b2 = abs1(h(k - 1, k - 1) - h(k, k));
                        const double aa = fmax(b1, b2), bb = fmin(b1, b2);
                        const double sab = aa + ab;
                        if (ba * (ab / sab) <= fmax(smlnum, ulp * (bb * (aa / sab)))) break;
                    }
                }
                if (k > ilo) h(k, k - 1) = mk(0.0);
                q.l = k;
                if (k < i) {
                    const int kd = kdefl + 1;
                    zc t;
                    if (kd % (2 * KEXSH) == 0) {
                        t = h(i, i) + 0.75 * fabs(h(i, i - 1).re);
                    } else if (kd % KEXSH == 0) {
                        t = h(k, k) + 0.75 * fabs(h(k + 1, k).re);
                    } else {  // Wilkinson's shift
                        t = h(i, i);
                        const zc u = zsqrt(h(i - 1, i)) * zsqrt(h(i, i - 1));
                        double s = abs1(u);
                        if (s != 0.0) {
                            const zc x = 0.5 * (h(i - 1, i - 1) - t);
                            const double sx = abs1(x);
                            s = fmax(s, sx);
                            const zc xs = x / s, us = u / s;
                            zc y = s * zsqrt(xs * xs + us * us);
                            if (sx > 0.0) {
                                const zc xn = x / sx;
                                if (xn.re * y.re + xn.im * y.im < 0.0) y = -y;
                            }
                            t = t - u * (u / (x + y));
                        }
                    }
                    // two consecutive small subdiagonal elements: start the sweep at row m
                    int m;
                    for (m = i - 1; m > k; --m) {
                        const zc h11 = h(m, m), h22 = h(m + 1, m + 1);
                        zc h11s = h11 - t;
                        double h21 = h(m + 1, m).re;
                        const double s = abs1(h11s) + fabs(h21);
                        h11s = h11s / s;
                        h21 /= s;
                        v0 = h11s;
                        v1 = mk(h21);
                        const double h10 = h(m, m - 1).re;
                        if (fabs(h10) * fabs(h21) <= ulp * (abs1(h11s) * (abs1(h11) + abs1(h22)))) break;
                    }
                    if (m == k) {
                        const zc h11s = h(k, k) - t;
                        const double h21 = h(k + 1, k).re;
                        const double s = abs1(h11s) + fabs(h21);
                        v0 = h11s / s;
                        v1 = mk(h21 / s);
                    }
                    q.m = m;
                }
            }
            __syncthreads();
            l = q.l;
            if (l >= i) {
                done = true;
                break;
            }
            ++kdefl;
            const int i1 = l, i2 = i, m = q.m;
            // the single-shift QR sweep
            for (int kk = m; kk < i; ++kk) {
                if (tid == 0) {
                    if (kk > m) {
                        v0 = h(kk, kk - 1);
                        v1 = h(kk + 1, kk - 1);
                    }
                    const zc t1 = larfg2(v0, v1);
                    if (kk > m) {
                        h(kk, kk - 1) = v0;
                        h(kk + 1, kk - 1) = mk(0.0);
                    }
                    q.t1 = t1;
                    q.v2 = v1;
                    q.t2 = (t1 * v1).re;
                }
                __syncthreads();
                const zc t1 = q.t1, v2 = q.v2;
                const double t2 = q.t2;
                // from the left: rows kk, kk+1, columns kk..i2
                const zc ct1 = conjz(t1);
                for (int j = kk + tid; j <= i2; j += NT) {
                    const zc sum = ct1 * h(kk, j) + t2 * h(kk + 1, j);
                    h(kk, j) -= sum;
                    h(kk + 1, j) -= sum * v2;
                }
                __syncthreads();
                // from the right: columns kk, kk+1, rows i1..min(kk+2, i)
                const zc cv2 = conjz(v2);
                const int jt = min(kk + 2, i);
                for (int j = i1 + tid; j <= jt; j += NT) {
                    const zc sum = t1 * h(j, kk) + t2 * h(j, kk + 1);
                    h(j, kk) -= sum;
                    h(j, kk + 1) -= sum * cv2;
                }
                if (kk == m && m > l) {
                    // the sweep started below l: keep H(m, m-1) real.  Row j in S =
                    // [m, i] \ {m+1} takes temp right of the diagonal, column j in S takes
                    // conj(temp) above it (zlahqr, one row and column at a time); an
                    // entry in both keeps its value
                    zc temp = 1.0 - t1;
                    temp = temp / zabs(temp);
                    __syncthreads();
                    if (tid == 0) {
                        h(m + 1, m) = h(m + 1, m) * conjz(temp);
                        if (m + 2 <= i) h(m + 2, m + 1) = h(m + 2, m + 1) * temp;
                    }
                    auto in_s = [&](int x) { return x >= m && x <= i && x != m + 1; };
                    const int na = i - i1 + 1;
                    for (int e = tid; e < na * na; e += NT) {
                        const int r = i1 + e % na, c = i1 + e / na;
                        if (r >= c) continue;
                        const bool a = in_s(r), b = in_s(c);
                        if (a && !b) h(r, c) = h(r, c) * temp;
                        else if (b && !a) h(r, c) = h(r, c) * conjz(temp);
                    }
                }
                __syncthreads();
            }
            // H(i, i-1) made real
            if (tid == 0) {
                const zc temp = h(i, i - 1);
                q.flag = temp.im != 0.0;
                if (q.flag) {
                    const double rt = zabs(temp);
                    q.temp = temp / rt;
                    h(i, i - 1) = mk(rt);
                }
            }
            __syncthreads();
            if (q.flag) {
                const zc u = q.temp;
                for (int c = i + 1 + tid; c <= i2; c += NT) h(i, c) = h(i, c) * conjz(u);
                for (int r = i1 + tid; r < i; r += NT) h(r, i) = h(r, i) * u;
            }
            __syncthreads();
        }
        if (!done) return i + 1;
        if (tid == 0) w[i] = h(i, i);
        kdefl = 0;
        i = l - 1;
    }
    return 0;
}

__global__ void __launch_bounds__(NT, 2) k_eigvals(EigParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LuSmem& s = *reinterpret_cast<LuSmem*>(smem_raw);
    __shared__ HqrShared q;
    zc* A = P.work + (size_t)blockIdx.x * P.slot;
    for (int it = blockIdx.x; it < P.nitem; it += gridDim.x) {
        const int n = P.item_n[it];
        const zc k = mk(P.ks[2 * it], P.ks[2 * it + 1]);
        assemble(A, nullptr, n, P.item_d[it], P.pos + P.item_pos[it], P.item_model[it], k, s);
        __syncthreads();
        if (P.normalized) {
            // build_normalized_matrix (ms_matrix_util.c:50): off the diagonal -G(k, r_ij) / I(k, 0),
            // that is M_ij / I(k, 0); i on the diagonal
            if (threadIdx.x == 0) s.diag[0] = free_green_imag(P.item_d[it], k, 0.0);
            __syncthreads();
            const zc iz = s.diag[0];
            for (size_t e = threadIdx.x; e < (size_t)n * n; e += NT) {
                const size_t r = e % n, c = e / n;
                A[e] = r == c ? mk(0.0, 1.0) : A[e] / iz;
            }
            __syncthreads();
        }
        if (P.trg2) {
            // tracegtwo (ms_matrix_util.c:167): 2 sum_{i<j} |A_ij|^2 / n, the matrix symmetric
            double t = 0.0, z1 = 0.0, z2 = 0.0;
            for (size_t e = threadIdx.x; e < (size_t)n * n; e += NT)
                if (e % n < e / n) t += zabs2(A[e]);
            block_sum3(t, z1, z2, s);
            if (threadIdx.x == 0) P.trg2[it] = 2.0 * t / n;
        }
        hessenberg(A, n, s);
        const int info = hqr_cta(A, n, P.mu + P.item_out[it], q);
        if (threadIdx.x == 0) P.status[it] = info > 0 ? MSGPU_S_NOCONV : 0;
        __syncthreads();
    }
}

}  // namespace msg

namespace {
std::mutex g_eig_mu;
}

extern "C" int msgpu_eigvals_batch_mtype(int mtype, int nmed, const msgpu_medium* media, int nitem,
                                         const int* item_med, const double* ks, double* mu, int* status,
                                         double* trg2) {
    using namespace msg;
    if ((mtype != MSGPU_MTYPE_MSMATRIX && mtype != MSGPU_MTYPE_NORMALIZED) || nmed < 1 || !media || nitem < 1 || !ks ||
        !mu)
        return record_error(MSGPU_E_ARG, "eigvals: bad argument (mtype 0 or 1, nmed >= 1, nitem >= 1, non-null pointers)");
    int nmax = 0;
    size_t npos = 0;
    std::vector<size_t> med_pos(nmed);
    for (int m = 0; m < nmed; ++m) {
        if (media[m].n < 1 || media[m].d < 1 || !media[m].pos)
            return record_error(MSGPU_E_ARG, "eigvals: a medium has n < 1, d < 1 or no positions");
        nmax = std::max(nmax, media[m].n);
        med_pos[m] = npos;
        npos += (size_t)media[m].n * media[m].d;
    }
    if (nmax > EIG_NMAX) return record_error(MSGPU_E_SIZE, "eigvals: n > 4097 (the reflector lives in shared memory)");
    for (int i = 0; i < nitem; ++i)
        if (item_med && (item_med[i] < 0 || item_med[i] >= nmed))
            return record_error(MSGPU_E_ARG, "eigvals: item_med out of range");
    const int sms = msgpu_sm_count();  // initialises the device and the kernels' attributes
    if (sms < 1) return record_error(MSGPU_E_NODEV, "eigvals: no CUDA device");
    std::lock_guard<std::mutex> lk(g_eig_mu);
    // on every call: the attribute belongs to the current device
    if (cudaFuncSetAttribute(k_eigvals, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LuSmem)) !=
        cudaSuccess)
        return record_error(MSGPU_E_CUDA, "eigvals: cudaFuncSetAttribute (shared memory) failed");
    std::vector<int> hn(nitem), hd(nitem);
    std::vector<size_t> hpos(nitem), hout(nitem);
    std::vector<msgpu_model> hmodel(nitem);
    size_t nout = 0;
    for (int i = 0; i < nitem; ++i) {
        const int mi = item_med ? item_med[i] : 0;
        hn[i] = media[mi].n;
        hd[i] = media[mi].d;
        hpos[i] = med_pos[mi];
        hmodel[i] = media[mi].model;
        hout[i] = nout;
        nout += (size_t)media[mi].n;
    }
    const size_t slot = (size_t)nmax * nmax;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return record_error(MSGPU_E_CUDA, "eigvals: cudaMemGetInfo failed");
    const size_t budget = free_b > ((size_t)4 << 30) ? free_b - ((size_t)4 << 30) : free_b / 2;
    const int grid = (int)std::min<size_t>({(size_t)nitem, (size_t)2 * sms, std::max<size_t>(1, budget / (slot * 16))});
    double *dpos = nullptr, *dks = nullptr;
    zc *dmu = nullptr, *dwork = nullptr;
    int *dn = nullptr, *dd = nullptr, *dst = nullptr;
    double* dtrg = nullptr;
    size_t *dposo = nullptr, *douto = nullptr;
    msgpu_model* dmodel = nullptr;
    auto cleanup = [&]() {
        cudaFree(dpos); cudaFree(dks); cudaFree(dmu); cudaFree(dwork); cudaFree(dn); cudaFree(dd);
        cudaFree(dst); cudaFree(dposo); cudaFree(douto); cudaFree(dmodel); cudaFree(dtrg);
    };
    if (cudaMalloc(&dpos, sizeof(double) * npos) || cudaMalloc(&dks, sizeof(double) * 2 * nitem) ||
        cudaMalloc(&dmu, sizeof(zc) * nout) || cudaMalloc(&dwork, sizeof(zc) * slot * grid) ||
        cudaMalloc(&dn, sizeof(int) * nitem) || cudaMalloc(&dd, sizeof(int) * nitem) ||
        cudaMalloc(&dst, sizeof(int) * nitem) || cudaMalloc(&dposo, sizeof(size_t) * nitem) ||
        cudaMalloc(&douto, sizeof(size_t) * nitem) || cudaMalloc(&dmodel, sizeof(msgpu_model) * nitem) ||
        (trg2 && cudaMalloc(&dtrg, sizeof(double) * nitem))) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "eigvals: device allocation failed");
    }
    bool ok = true;
    for (int m = 0; m < nmed && ok; ++m)
        ok = cudaMemcpy(dpos + med_pos[m], media[m].pos, sizeof(double) * (size_t)media[m].n * media[m].d,
                        cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemcpy(dks, ks, sizeof(double) * 2 * nitem, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(dn, hn.data(), sizeof(int) * nitem, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(dd, hd.data(), sizeof(int) * nitem, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(dposo, hpos.data(), sizeof(size_t) * nitem, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(douto, hout.data(), sizeof(size_t) * nitem, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(dmodel, hmodel.data(), sizeof(msgpu_model) * nitem, cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemset(dmu, 0, sizeof(zc) * nout) == cudaSuccess;  // unconverged values read 0
    if (!ok) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "eigvals: host-to-device copy failed");
    }
    EigParams P{nitem, dn, dd, dposo, dmodel, dpos, dks, douto, dmu, dst, dwork, slot,
                mtype == MSGPU_MTYPE_NORMALIZED, dtrg};
    k_eigvals<<<grid, NT, sizeof(LuSmem)>>>(P);
    count_launches(1);
    std::vector<int> hst(nitem);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(mu, dmu, sizeof(zc) * nout, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hst.data(), dst, sizeof(int) * nitem, cudaMemcpyDeviceToHost) != cudaSuccess ||
        (trg2 && cudaMemcpy(trg2, dtrg, sizeof(double) * nitem, cudaMemcpyDeviceToHost) != cudaSuccess)) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "eigvals: kernel launch, execution or device-to-host copy failed");
    }
    if (status)
        for (int i = 0; i < nitem; ++i) status[i] = hst[i];
    cleanup();
    return 0;
}

extern "C" int msgpu_eigvals_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med,
                                   const double* ks, double* mu, int* status) {
    return msgpu_eigvals_batch_mtype(MSGPU_MTYPE_MSMATRIX, nmed, media, nitem, item_med, ks, mu, status, nullptr);
}
