// wave.cu -- wavefunction on a pixel grid (reference run_wave_function_omp,
// src/core/ms_core.c:596-649): a = M^-1 phi for a plane wave along +x, then
// psi(r) = exp(i k x) + sum_i a_i G(k, |r - x_i|) (eval_total_wave,
// src/core/incident_wave_util.c:87-96) at every pixel of an nx x ny grid of
// the (x, y, 0...) plane, row-major from (xmin, ymax) (get_pos_wfun,
// src/core/wave_function_util.c:76-81).  Averaged over media (seeds): the
// real part and |psi|^2, as the reference accumulates them.
//
// Several wave numbers at once: every (medium, k) solve goes into one
// amplitude job (one persistent engine launch), then one grid launch per
// medium covers every k (blockIdx.y), accumulating into per-k planes.
//
// One thread per pixel; atoms stream through shared memory in tiles of 256.
//   FP64 kernel : the reference's arithmetic, bound by the FP64 pipe.
//   DF kernel   : d = 3 only, the Green function in double-float arithmetic
//                 on the FP32 pipe (green_df.cuh), used by the mixed precision
//                 when |Im k| * r stays below 80 over the grid.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <vector>
#include "msgpu.h"
#include "green.cuh"
#include "green_df.cuh"
#include "engine_internal.h"

namespace msg {

constexpr int PT = 256;

struct GridArgs {
    int d, n, nx, ny;
    const double* pos;
    const double* amp;  // [nk][n] complex
    const double* ks;   // [nk] complex
    double xmin, dx, ymax, dy;
    double* fun;  // [nk][nx*ny]
    double* den;
    double* psi;  // [nk][nx*ny] complex, or null
};

__device__ __forceinline__ void finish_pixel(const GridArgs& A, int kk, int l, double px, zc acc) {
    const size_t o = (size_t)kk * A.nx * A.ny + l;
    const zc k = mk(A.ks[2 * kk], A.ks[2 * kk + 1]);
    const zc v = acc + zexp(mk(0.0, 1.0) * k * px);
    A.fun[o] += v.re;
    A.den[o] += v.re * v.re + v.im * v.im;
    if (A.psi) {
        A.psi[2 * o] = v.re;
        A.psi[2 * o + 1] = v.im;
    }
}

__global__ void __launch_bounds__(PT) k_psi_grid(GridArgs A) {
    __shared__ double sx[PT], sy[PT], sr[PT], sar[PT], sai[PT];
    const int kk = blockIdx.y;
    const int l = blockIdx.x * PT + threadIdx.x;
    const bool live = l < A.nx * A.ny;
    const double px = A.xmin + (l % A.nx) * A.dx, py = A.ymax - (l / A.nx) * A.dy;
    const zc k = mk(A.ks[2 * kk], A.ks[2 * kk + 1]);
    const double* amp = A.amp + 2 * (size_t)kk * A.n;
    zc acc = mk(0.0);
    for (int t0 = 0; t0 < A.n; t0 += PT) {
        const int i = t0 + threadIdx.x;
        if (i < A.n) {
            const double* p = A.pos + (size_t)i * A.d;
            sx[threadIdx.x] = p[0];
            sy[threadIdx.x] = A.d > 1 ? p[1] : 0.0;
            double rest = 0.0;
            for (int c = 2; c < A.d; ++c) rest += p[c] * p[c];
            sr[threadIdx.x] = rest;
            sar[threadIdx.x] = amp[2 * i];
            sai[threadIdx.x] = amp[2 * i + 1];
        }
        __syncthreads();
        const int cnt = min(PT, A.n - t0);
        if (live) {
            for (int j = 0; j < cnt; ++j) {
                const double ex = sx[j] - px, ey = sy[j] - py;
                const double r = sqrt(ex * ex + ey * ey + sr[j]);
                acc += mk(sar[j], sai[j]) * free_green(A.d, k, r);
            }
        }
        __syncthreads();
    }
    if (live) finish_pixel(A, kk, l, px, acc);
}

__global__ void __launch_bounds__(PT) k_psi_grid_df3(GridArgs A) {
    __shared__ Df3Tables tab;
    __shared__ float4 sxy[PT];  // x.h x.l y.h y.l
    __shared__ float2 sz[PT];   // z^2 (d = 3)
    __shared__ float4 sa[PT];   // a as double-float complex
    df3_tables_init(tab);
    const int kk = blockIdx.y;
    const int l = blockIdx.x * PT + threadIdx.x;
    const bool live = l < A.nx * A.ny;
    const double pxd = A.xmin + (l % A.nx) * A.dx, pyd = A.ymax - (l / A.nx) * A.dy;
    const df px = df_from_double(pxd), py = df_from_double(pyd);
    const df kr = df_from_double(A.ks[2 * kk]), ki = df_from_double(A.ks[2 * kk + 1]);
    const bool grow = A.ks[2 * kk + 1] != 0.0;
    const double* amp = A.amp + 2 * (size_t)kk * A.n;
    dfc acc{df{0.0f, 0.0f}, df{0.0f, 0.0f}};
    for (int t0 = 0; t0 < A.n; t0 += PT) {
        const int i = t0 + threadIdx.x;
        if (i < A.n) {
            const double* p = A.pos + (size_t)i * 3;
            const df x = df_from_double(p[0]), y = df_from_double(p[1]), z2 = df_from_double(p[2] * p[2]);
            sxy[threadIdx.x] = make_float4(x.h, x.l, y.h, y.l);
            sz[threadIdx.x] = make_float2(z2.h, z2.l);
            const df ar = df_from_double(amp[2 * i]), ai = df_from_double(amp[2 * i + 1]);
            sa[threadIdx.x] = make_float4(ar.h, ar.l, ai.h, ai.l);
        }
        __syncthreads();
        const int cnt = min(PT, A.n - t0);
        if (live) {
            for (int j = 0; j < cnt; ++j) {
                const float4 q = sxy[j];
                const float2 z = sz[j];
                const df ex = df_sub(df{q.x, q.y}, px), ey = df_sub(df{q.z, q.w}, py);
                const df r2 = df_add(df_add(df_mul(ex, ex), df_mul(ey, ey)), df{z.x, z.y});
                const float4 a = sa[j];
                df3_green_mac(tab, kr, ki, grow, df_sqrt(r2), dfc{df{a.x, a.y}, df{a.z, a.w}}, acc);
            }
        }
        __syncthreads();
    }
    if (live) finish_pixel(A, kk, l, pxd, mk(df_to_double(acc.re), df_to_double(acc.im)));
}

}  // namespace msg

extern "C" int msgpu_wave_function_batch(int nmed, const msgpu_medium* media, int nk, const double* ks, int nx,
                                         int ny, const double* dom, double* function, double* density, double* psi,
                                         double* amps, int precision) {
    using namespace msg;
    if (nmed < 1 || !media || nk < 1 || !ks || nx < 2 || ny < 2 || !dom || !function || !density)
        return record_error(MSGPU_E_ARG,
                            "wave_function: bad argument (nmed, nk >= 1; nx, ny >= 2; non-null pointers)");
    const int n = media[0].n, d = media[0].d;
    for (int m = 0; m < nmed; ++m)
        if (media[m].n != n || media[m].d != d || !media[m].pos)
            return record_error(MSGPU_E_ARG,
                                "wave_function: every medium needs the same n and d, and positions");
    const size_t np = (size_t)nx * ny;
    if (np > (size_t)1 << 31 || (size_t)nk > 65535)
        return record_error(MSGPU_E_SIZE,
                            "wave_function: more than 2^31 pixels or 65535 wave numbers");
    // every (medium, k) solve in one job: item m * nk + kk
    const int nitem = nmed * nk;
    std::vector<double> iks(2 * (size_t)nitem), sig(2 * (size_t)nitem), a(2 * (size_t)nitem * n);
    std::vector<int> im(nitem), st(nitem);
    for (int m = 0; m < nmed; ++m)
        for (int kk = 0; kk < nk; ++kk) {
            const int it = m * nk + kk;
            iks[2 * it] = ks[2 * kk];
            iks[2 * it + 1] = ks[2 * kk + 1];
            im[it] = m;
        }
    int e = msgpu_amplitude_batch(nmed, media, nitem, im.data(), iks.data(), sig.data(), a.data(), st.data(),
                                  precision);
    if (e) return e;
    if (amps) std::copy(a.begin(), a.end(), amps);
    // the double-float Green function keeps values in FP32 range: |Im k| * r < 80
    double rmax = 0.0, kimax = 0.0;
    for (int kk = 0; kk < nk; ++kk) kimax = std::max(kimax, std::fabs(ks[2 * kk + 1]));
    if (d == 3 && precision == MSGPU_MIXED) {
        double lo[3] = {dom[0], dom[2], 0.0}, hi[3] = {dom[1], dom[3], 0.0};
        for (int m = 0; m < nmed; ++m)
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < 3; ++c) {
                    lo[c] = std::min(lo[c], media[m].pos[3 * i + c]);
                    hi[c] = std::max(hi[c], media[m].pos[3 * i + c]);
                }
        rmax = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                         (hi[2] - lo[2]) * (hi[2] - lo[2]));
    }
    const bool use_df = d == 3 && precision == MSGPU_MIXED && kimax * rmax < 80.0;
    double *dpos = nullptr, *damp = nullptr, *dks = nullptr, *dfun = nullptr, *dden = nullptr, *dpsi = nullptr;
    auto cleanup = [&]() {
        cudaFree(dpos); cudaFree(damp); cudaFree(dks); cudaFree(dfun); cudaFree(dden); cudaFree(dpsi);
    };
    const size_t plane = np * nk;
    if (cudaMalloc(&dpos, sizeof(double) * (size_t)n * d) || cudaMalloc(&damp, sizeof(double) * 2 * (size_t)nk * n) ||
        cudaMalloc(&dks, sizeof(double) * 2 * nk) || cudaMalloc(&dfun, sizeof(double) * plane) ||
        cudaMalloc(&dden, sizeof(double) * plane) || (psi && cudaMalloc(&dpsi, sizeof(double) * 2 * plane))) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "wave_function: device allocation failed");
    }
    if (cudaMemset(dfun, 0, sizeof(double) * plane) || cudaMemset(dden, 0, sizeof(double) * plane) ||
        cudaMemcpy(dks, ks, sizeof(double) * 2 * nk, cudaMemcpyHostToDevice)) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "wave_function: upload to the device failed");
    }
    GridArgs A;
    A.d = d;
    A.n = n;
    A.nx = nx;
    A.ny = ny;
    A.pos = dpos;
    A.amp = damp;
    A.ks = dks;
    A.xmin = dom[0];
    A.dx = (dom[1] - dom[0]) / (nx - 1);
    A.ymax = dom[3];
    A.dy = (dom[3] - dom[2]) / (ny - 1);
    A.fun = dfun;
    A.den = dden;
    const dim3 grid((unsigned)((np + PT - 1) / PT), (unsigned)nk);
    for (int m = 0; m < nmed; ++m) {
        if (cudaMemcpy(dpos, media[m].pos, sizeof(double) * (size_t)n * d, cudaMemcpyHostToDevice) ||
            cudaMemcpy(damp, a.data() + 2 * (size_t)m * nk * n, sizeof(double) * 2 * (size_t)nk * n,
                       cudaMemcpyHostToDevice)) {
            cleanup();
            return record_error(MSGPU_E_CUDA, "wave_function: upload to the device failed");
        }
        A.psi = m == 0 ? dpsi : nullptr;
        if (use_df) k_psi_grid_df3<<<grid, PT>>>(A);
        else k_psi_grid<<<grid, PT>>>(A);
        count_launches(1);
        if (cudaGetLastError() != cudaSuccess) {
            cleanup();
            return record_error(MSGPU_E_CUDA, "wave_function: kernel launch failed");
        }
    }
    cudaError_t ce = cudaMemcpy(function, dfun, sizeof(double) * plane, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(density, dden, sizeof(double) * plane, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && psi) ce = cudaMemcpy(psi, dpsi, sizeof(double) * 2 * plane, cudaMemcpyDeviceToHost);
    cleanup();
    if (ce != cudaSuccess) return record_error(MSGPU_E_CUDA, "wave_function: copy of the results to the host failed");
    // divide_wfun (wave_function_util.c:86): average over the realisations
    for (size_t l = 0; l < plane; ++l) {
        function[l] /= nmed;
        density[l] /= nmed;
    }
    // the solves' status words, OR-ed: a singular or non-finite solve reached the averages
    int any = 0;
    for (int v : st) any |= v;
    return any;
}

// Seed-averaged wavefunction of run_wave_function_omp at one wave number k.
extern "C" int msgpu_wave_function(int nmed, const msgpu_medium* media, const double* k, int nx, int ny,
                                   const double* dom, double* function, double* density, double* psi,
                                   double* amps, int precision) {
    return msgpu_wave_function_batch(nmed, media, 1, k, nx, ny, dom, function, density, psi, amps, precision);
}

// Wavefunction cut of run_wave_function_cut_omp (src/core/ms_core.c:654-703):
// every medium's amplitudes in one job, then psi at the nbin points
// (xmin + i dx, 0, ...) of the x axis (get_pos_wfcut, wave_function_cut_util.c:83,
// dx = (xmax - xmin)/(nbin - 1) as init_wfcut sets it) per medium: the grid
// kernel on a one-row grid, each medium writing its own row of psi.
extern "C" int msgpu_wave_cut(int nmed, const msgpu_medium* media, const double* k, int nbin, double xmin,
                              double xmax, double* psi, double* amps, int precision) {
    using namespace msg;
    if (nmed < 1 || !media || !k || nbin < 2 || !psi)
        return record_error(MSGPU_E_ARG,
                            "wave_cut: bad argument (nmed >= 1, nbin >= 2, non-null pointers)");
    const int n = media[0].n, d = media[0].d;
    for (int m = 0; m < nmed; ++m)
        if (media[m].n != n || media[m].d != d || !media[m].pos)
            return record_error(MSGPU_E_ARG,
                                "wave_cut: every medium needs the same n and d, and positions");
    if ((size_t)nmed * nbin > (size_t)1 << 31) return record_error(MSGPU_E_SIZE, "wave_cut: more than 2^31 samples");
    std::vector<double> iks(2 * (size_t)nmed), sig(2 * (size_t)nmed), a(2 * (size_t)nmed * n);
    std::vector<int> im(nmed), st(nmed);
    for (int m = 0; m < nmed; ++m) {
        iks[2 * m] = k[0];
        iks[2 * m + 1] = k[1];
        im[m] = m;
    }
    int e = msgpu_amplitude_batch(nmed, media, nmed, im.data(), iks.data(), sig.data(), a.data(), st.data(),
                                  precision);
    if (e) return e;
    if (amps) std::copy(a.begin(), a.end(), amps);
    // every medium's positions in one array; the double-float Green function needs |Im k| * r < 80
    std::vector<double> pos((size_t)nmed * n * d);
    double lo[3] = {std::min(xmin, xmax), 0.0, 0.0}, hi[3] = {std::max(xmin, xmax), 0.0, 0.0};
    for (int m = 0; m < nmed; ++m) {
        std::copy(media[m].pos, media[m].pos + (size_t)n * d, pos.begin() + (size_t)m * n * d);
        if (d == 3)
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < 3; ++c) {
                    lo[c] = std::min(lo[c], media[m].pos[3 * i + c]);
                    hi[c] = std::max(hi[c], media[m].pos[3 * i + c]);
                }
    }
    const double rmax = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                  (hi[2] - lo[2]) * (hi[2] - lo[2]));
    const bool use_df = d == 3 && precision == MSGPU_MIXED && std::fabs(k[1]) * rmax < 80.0;
    double *dpos = nullptr, *damp = nullptr, *dks = nullptr, *dfun = nullptr, *dden = nullptr, *dpsi = nullptr;
    auto cleanup = [&]() {
        cudaFree(dpos); cudaFree(damp); cudaFree(dks); cudaFree(dfun); cudaFree(dden); cudaFree(dpsi);
    };
    const size_t rows = (size_t)nmed * nbin;
    if (cudaMalloc(&dpos, sizeof(double) * pos.size()) || cudaMalloc(&damp, sizeof(double) * a.size()) ||
        cudaMalloc(&dks, sizeof(double) * 2) || cudaMalloc(&dfun, sizeof(double) * nbin) ||
        cudaMalloc(&dden, sizeof(double) * nbin) || cudaMalloc(&dpsi, sizeof(double) * 2 * rows)) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "wave_cut: device allocation failed");
    }
    if (cudaMemcpy(dpos, pos.data(), sizeof(double) * pos.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(damp, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(dks, k, sizeof(double) * 2, cudaMemcpyHostToDevice) ||
        cudaMemset(dfun, 0, sizeof(double) * nbin) || cudaMemset(dden, 0, sizeof(double) * nbin)) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "wave_cut: upload to the device failed");
    }
    GridArgs A;
    A.d = d;
    A.n = n;
    A.nx = nbin;
    A.ny = 1;
    A.ks = dks;
    A.xmin = xmin;
    A.dx = (xmax - xmin) / (nbin - 1);
    A.ymax = 0.0;
    A.dy = 0.0;
    A.fun = dfun;  // the grid kernels' sums over media, not read
    A.den = dden;
    const dim3 grid((unsigned)((nbin + PT - 1) / PT), 1u);
    for (int m = 0; m < nmed; ++m) {
        A.pos = dpos + (size_t)m * n * d;
        A.amp = damp + 2 * (size_t)m * n;
        A.psi = dpsi + 2 * (size_t)m * nbin;
        if (use_df) k_psi_grid_df3<<<grid, PT>>>(A);
        else k_psi_grid<<<grid, PT>>>(A);
        count_launches(1);
        if (cudaGetLastError() != cudaSuccess) {
            cleanup();
            return record_error(MSGPU_E_CUDA, "wave_cut: kernel launch failed");
        }
    }
    const cudaError_t ce = cudaMemcpy(psi, dpsi, sizeof(double) * 2 * rows, cudaMemcpyDeviceToHost);
    cleanup();
    if (ce != cudaSuccess) return record_error(MSGPU_E_CUDA, "wave_cut: copy of the results to the host failed");
    int any = 0;
    for (int v : st) any |= v;
    return any;
}

namespace msg {

constexpr int FF_NT = 128;

// Far-field amplitude of run_differential_cross_section_omp (ms_core.c:556-562):
// for medium m = blockIdx.y and angle i = blockIdx.x, atot = sum_j conj(b_j) a_j
// with b_j = exp(i k (cos th x_j + sin th y_j)) (build_plane_wave,
// ms_matrix_util.c:88-107; d = 1: exp(i k sign(cos th) x_j)) and real k, so
// conj(b_j) = cos(k u_j) - i sin(k u_j); out[m + i*nmed] = prefac |atot|^2.
__global__ void __launch_bounds__(FF_NT) k_far_field(int d, int n, int nmed, double k, const double* __restrict__ pos,
                                                     const double* __restrict__ amp, const double* __restrict__ cs,
                                                     double prefac, double* __restrict__ out) {
    __shared__ double red[2][FF_NT / 32];
    const int i = blockIdx.x, m = blockIdx.y;
    const double ct = cs[2 * i], st = cs[2 * i + 1];
    const double* p = pos + (size_t)m * n * d;
    const double* a = amp + 2 * (size_t)m * n;
    double re = 0.0, im = 0.0;
    for (int j = threadIdx.x; j < n; j += FF_NT) {
        const double u = d == 1 ? (ct > 0.0 ? 1.0 : -1.0) * p[j] : ct * p[(size_t)j * d] + st * p[(size_t)j * d + 1];
        double s, c;
        sincos(k * u, &s, &c);
        const double ar = a[2 * j], ai = a[2 * j + 1];
        re += c * ar + s * ai;  // (c - i s)(ar + i ai)
        im += c * ai - s * ar;
    }
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = re;
        red[1][w] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0, q = 0.0;
        for (int v = 0; v < FF_NT / 32; ++v) {
            r += red[0][v];
            q += red[1][v];
        }
        out[(size_t)m + (size_t)i * nmed] = prefac * (r * r + q * q);
    }
}

}  // namespace msg

// Differential cross section of run_differential_cross_section_omp
// (src/core/ms_core.c:526-594) at real k: every medium's amplitudes in one job,
// then prefac |sum_j conj(b_j(th_i)) a_j|^2 for the nbin angles
// th_i = thmin exp(i log(thmax/thmin)/(nbin-1)) degrees (get_arg_dcs,
// diff_cross_section_util.c:86), prefac = (k/2pi)^(d-3)/(16 pi^2), into
// samples[m + i*nmed] (the reference's layout before its sort).
extern "C" int msgpu_diff_cross_section(int nmed, const msgpu_medium* media, double k, int nbin, double thmin,
                                        double thmax, double* samples, int precision) {
    using namespace msg;
    if (nmed < 1 || nmed > 65535 || !media || nbin < 2 || !samples || !(thmin > 0.0) || !(thmax > 0.0))
        return record_error(MSGPU_E_ARG,
                            "diff_cross_section: bad argument (1 <= nmed <= 65535, nbin >= 2, thmin and thmax > 0, "
                            "non-null pointers)");
    const int n = media[0].n, d = media[0].d;
    for (int m = 0; m < nmed; ++m)
        if (media[m].n != n || media[m].d != d || !media[m].pos)
            return record_error(MSGPU_E_ARG,
                                "diff_cross_section: every medium needs the same n and d, and positions");
    if ((size_t)nmed * nbin > (size_t)1 << 31)
        return record_error(MSGPU_E_SIZE,
                            "diff_cross_section: more than 2^31 samples");
    std::vector<double> iks(2 * (size_t)nmed), sig(2 * (size_t)nmed), a(2 * (size_t)nmed * n);
    std::vector<int> im(nmed), st(nmed);
    for (int m = 0; m < nmed; ++m) {
        iks[2 * m] = k;
        iks[2 * m + 1] = 0.0;
        im[m] = m;
    }
    int e = msgpu_amplitude_batch(nmed, media, nmed, im.data(), iks.data(), sig.data(), a.data(), st.data(),
                                  precision);
    if (e) return e;
    const double pi = 3.1415926535897932385;
    std::vector<double> cs(2 * (size_t)nbin);
    for (int i = 0; i < nbin; ++i) {
        double th = thmin * std::exp(i * std::log(thmax / thmin) / (nbin - 1));  // degrees
        th *= pi / 180;
        cs[2 * i] = std::cos(th);
        cs[2 * i + 1] = std::sin(th);
    }
    const double prefac = std::pow(k / (2 * pi), d - 3) / (16 * pi * pi);
    std::vector<double> pos((size_t)nmed * n * d);
    for (int m = 0; m < nmed; ++m)
        std::copy(media[m].pos, media[m].pos + (size_t)n * d, pos.begin() + (size_t)m * n * d);
    double *dpos = nullptr, *damp = nullptr, *dcs = nullptr, *dout = nullptr;
    auto cleanup = [&]() { cudaFree(dpos); cudaFree(damp); cudaFree(dcs); cudaFree(dout); };
    const size_t nout = (size_t)nmed * nbin;
    if (cudaMalloc(&dpos, sizeof(double) * pos.size()) || cudaMalloc(&damp, sizeof(double) * a.size()) ||
        cudaMalloc(&dcs, sizeof(double) * cs.size()) || cudaMalloc(&dout, sizeof(double) * nout)) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "diff_cross_section: device allocation failed");
    }
    if (cudaMemcpy(dpos, pos.data(), sizeof(double) * pos.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(damp, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(dcs, cs.data(), sizeof(double) * cs.size(), cudaMemcpyHostToDevice)) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "diff_cross_section: upload to the device failed");
    }
    k_far_field<<<dim3((unsigned)nbin, (unsigned)nmed), FF_NT>>>(d, n, nmed, k, dpos, damp, dcs, prefac, dout);
    count_launches(1);
    if (cudaGetLastError() != cudaSuccess) {
        cleanup();
        return record_error(MSGPU_E_CUDA, "diff_cross_section: kernel launch failed");
    }
    const cudaError_t ce = cudaMemcpy(samples, dout, sizeof(double) * nout, cudaMemcpyDeviceToHost);
    cleanup();
    if (ce != cudaSuccess)
        return record_error(MSGPU_E_CUDA,
                            "diff_cross_section: copy of the results to the host failed");
    int any = 0;
    for (int v : st) any |= v;
    return any;
}
