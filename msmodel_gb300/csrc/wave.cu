// wave.cu -- wavefunction on a pixel grid (reference run_wave_function_omp,
// src/core/ms_core.c:596-649): a = M^-1 phi for a plane wave along +x, then
// psi(r) = exp(i k x) + sum_i a_i G(k, |r - x_i|) (eval_total_wave,
// src/core/incident_wave_util.c:87-96) at every pixel of an nx x ny grid of
// the (x, y, 0...) plane, row-major from (xmin, ymax) (get_pos_wfun,
// src/core/wave_function_util.c:76-81).  Averaged over media (seeds): the
// real part and |psi|^2, as the reference accumulates them.
//
// One thread per pixel; atoms stream through shared memory in tiles of 256
// (x, y, squared remaining coordinates, a).  FP64 throughout: pixels x atoms
// Green evaluations, bound by the FP64 pipe.
#include <cuda_runtime.h>
#include <vector>
#include "msgpu.h"
#include "green.cuh"
#include "engine_internal.h"

namespace msg {

constexpr int PT = 256;

__global__ void __launch_bounds__(PT) k_psi_grid(int d, int n, const double* __restrict__ pos,
                                                 const double* __restrict__ amp, double kre, double kim, int nx,
                                                 int ny, double xmin, double dx, double ymax, double dy,
                                                 double* __restrict__ fun, double* __restrict__ den,
                                                 double* __restrict__ psi) {
    __shared__ double sx[PT], sy[PT], sr[PT], sar[PT], sai[PT];
    const int l = blockIdx.x * PT + threadIdx.x;
    const bool live = l < nx * ny;
    const double px = xmin + (l % nx) * dx, py = ymax - (l / nx) * dy;
    const zc k = mk(kre, kim);
    zc acc = mk(0.0);
    for (int t0 = 0; t0 < n; t0 += PT) {
        const int i = t0 + threadIdx.x;
        if (i < n) {
            const double* p = pos + (size_t)i * d;
            sx[threadIdx.x] = p[0];
            sy[threadIdx.x] = d > 1 ? p[1] : 0.0;
            double rest = 0.0;
            for (int c = 2; c < d; ++c) rest += p[c] * p[c];
            sr[threadIdx.x] = rest;
            sar[threadIdx.x] = amp[2 * i];
            sai[threadIdx.x] = amp[2 * i + 1];
        }
        __syncthreads();
        const int cnt = min(PT, n - t0);
        if (live) {
            for (int j = 0; j < cnt; ++j) {
                const double ex = sx[j] - px, ey = sy[j] - py;
                const double r = sqrt(ex * ex + ey * ey + sr[j]);
                const zc g = free_green(d, k, r);
                acc += mk(sar[j], sai[j]) * g;
            }
        }
        __syncthreads();
    }
    if (!live) return;
    const zc v = acc + zexp(mk(0.0, 1.0) * k * px);
    fun[l] += v.re;
    den[l] += v.re * v.re + v.im * v.im;
    if (psi) {
        psi[2 * l] = v.re;
        psi[2 * l + 1] = v.im;
    }
}

}  // namespace msg

// Seed-averaged wavefunction of run_wave_function_omp: media[m] are the
// realisations (all of the same n, d), k the incident wave number.
// function/density: nx*ny doubles (averaged Re psi and |psi|^2); psi (may be
// NULL): complex psi of media[0]; amps (may be NULL): a of every medium.
extern "C" int msgpu_wave_function(int nmed, const msgpu_medium* media, const double* k, int nx, int ny,
                                   const double* dom, double* function, double* density, double* psi,
                                   double* amps, int precision) {
    using namespace msg;
    if (nmed < 1 || !media || !k || nx < 2 || ny < 2 || !dom || !function || !density) return MSGPU_E_ARG;
    const int n = media[0].n, d = media[0].d;
    for (int m = 0; m < nmed; ++m)
        if (media[m].n != n || media[m].d != d) return MSGPU_E_ARG;
    std::vector<double> ks(2 * (size_t)nmed), sig(2 * (size_t)nmed), a(2 * (size_t)nmed * n);
    std::vector<int> im(nmed), st(nmed);
    for (int m = 0; m < nmed; ++m) {
        ks[2 * m] = k[0];
        ks[2 * m + 1] = k[1];
        im[m] = m;
    }
    int e = msgpu_amplitude_batch(nmed, media, nmed, im.data(), ks.data(), sig.data(), a.data(), st.data(), precision);
    if (e) return e;
    if (amps) std::copy(a.begin(), a.end(), amps);
    const size_t np = (size_t)nx * ny;
    double *dpos = nullptr, *damp = nullptr, *dfun = nullptr, *dden = nullptr, *dpsi = nullptr;
    auto cleanup = [&]() {
        cudaFree(dpos); cudaFree(damp); cudaFree(dfun); cudaFree(dden); cudaFree(dpsi);
    };
    if (cudaMalloc(&dpos, sizeof(double) * (size_t)n * d) || cudaMalloc(&damp, sizeof(double) * 2 * (size_t)n) ||
        cudaMalloc(&dfun, sizeof(double) * np) || cudaMalloc(&dden, sizeof(double) * np) ||
        (psi && cudaMalloc(&dpsi, sizeof(double) * 2 * np))) {
        cleanup();
        return MSGPU_E_CUDA;
    }
    cudaMemset(dfun, 0, sizeof(double) * np);
    cudaMemset(dden, 0, sizeof(double) * np);
    const double dx = (dom[1] - dom[0]) / (nx - 1), dy = (dom[3] - dom[2]) / (ny - 1);
    const unsigned blocks = (unsigned)((np + PT - 1) / PT);
    for (int m = 0; m < nmed; ++m) {
        cudaMemcpy(dpos, media[m].pos, sizeof(double) * (size_t)n * d, cudaMemcpyHostToDevice);
        cudaMemcpy(damp, a.data() + 2 * (size_t)m * n, sizeof(double) * 2 * (size_t)n, cudaMemcpyHostToDevice);
        k_psi_grid<<<blocks, PT>>>(d, n, dpos, damp, k[0], k[1], nx, ny, dom[0], dx, dom[3], dy, dfun, dden,
                                   m == 0 ? dpsi : nullptr);
        count_launches(1);
        if (cudaGetLastError() != cudaSuccess) {
            cleanup();
            return MSGPU_E_CUDA;
        }
    }
    std::vector<double> hf(np), hd(np);
    cudaError_t ce = cudaMemcpy(hf.data(), dfun, sizeof(double) * np, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(hd.data(), dden, sizeof(double) * np, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && psi) ce = cudaMemcpy(psi, dpsi, sizeof(double) * 2 * np, cudaMemcpyDeviceToHost);
    cleanup();
    if (ce != cudaSuccess) return MSGPU_E_CUDA;
    // divide_wfun (wave_function_util.c:86): average over the realisations
    for (size_t l = 0; l < np; ++l) {
        function[l] = hf[l] / nmed;
        density[l] = hd[l] / nmed;
    }
    return 0;
}
