// eigvals.cu -- the eigenvalues mu of M(k), the input of the reference's
// mu-plane histograms (eigvals, src/core/ms_matrix_util.c:147, zgeev_ without
// eigenvectors; run_chistogram_omp and run_imag_mu_histogram_omp,
// src/core/ms_core.c:173-282).  This is not the hot path: M(k) is assembled
// on the GPU by this library's kernel, and the general complex eigenproblem
// (Hessenberg reduction and shifted QR) is handed to cuSOLVER's Xgeev, one
// matrix after another on one stream.
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include "msgpu.h"
#include "lu64.cuh"
#include "engine_internal.h"

namespace msg {
__global__ void __launch_bounds__(NT, 1) k_build_matrix(zc* A, int n, int d, const double* pos, msgpu_model m,
                                                        double kre, double kim, int deriv);
}  // namespace msg

namespace {
std::mutex g_eig_mu;
cusolverDnHandle_t g_solver = nullptr;
cusolverDnParams_t g_params = nullptr;
}  // namespace

extern "C" int msgpu_eigvals_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med,
                                   const double* ks, double* mu, int* status) {
    using namespace msg;
    if (nmed < 1 || !media || nitem < 1 || !ks || !mu) return MSGPU_E_ARG;
    int nmax = 0;
    for (int m = 0; m < nmed; ++m) {
        if (media[m].n < 1 || media[m].d < 1 || !media[m].pos) return MSGPU_E_ARG;
        nmax = std::max(nmax, media[m].n);
    }
    for (int i = 0; i < nitem; ++i)
        if (item_med && (item_med[i] < 0 || item_med[i] >= nmed)) return MSGPU_E_ARG;
    const int sms = msgpu_sm_count();  // initialises the device and the kernels' attributes
    if (sms < 1) return MSGPU_E_NODEV;
    std::lock_guard<std::mutex> lk(g_eig_mu);
    if (!g_solver && (cusolverDnCreate(&g_solver) != CUSOLVER_STATUS_SUCCESS ||
                      cusolverDnCreateParams(&g_params) != CUSOLVER_STATUS_SUCCESS))
        return MSGPU_E_CUDA;
    double* dpos = nullptr;
    zc *dA = nullptr, *dW = nullptr;
    int* dinfo = nullptr;
    void* dwork = nullptr;
    size_t dwork_bytes = 0;
    std::vector<char> hwork;
    auto cleanup = [&]() {
        cudaFree(dpos); cudaFree(dA); cudaFree(dW); cudaFree(dinfo); cudaFree(dwork);
    };
    size_t npos = 0;
    for (int m = 0; m < nmed; ++m) npos = std::max(npos, (size_t)media[m].n * media[m].d);
    if (cudaMalloc(&dpos, sizeof(double) * npos) || cudaMalloc(&dA, sizeof(zc) * (size_t)nmax * nmax) ||
        cudaMalloc(&dW, sizeof(zc) * (size_t)nmax) || cudaMalloc(&dinfo, sizeof(int))) {
        cleanup();
        return MSGPU_E_CUDA;
    }
    size_t off = 0;
    int last_med = -1;
    for (int it = 0; it < nitem; ++it) {
        const int mi = item_med ? item_med[it] : 0;
        const msgpu_medium& md = media[mi];
        const int n = md.n;
        if (mi != last_med) {
            if (cudaMemcpy(dpos, md.pos, sizeof(double) * (size_t)n * md.d, cudaMemcpyHostToDevice)) {
                cleanup();
                return MSGPU_E_CUDA;
            }
            last_med = mi;
        }
        const int nt = (n + 31) / 32;
        k_build_matrix<<<std::min(nt, 4 * sms), NT, sizeof(LuSmem)>>>(dA, n, md.d, dpos, md.model, ks[2 * it],
                                                                      ks[2 * it + 1], 0);
        count_launches(1);
        size_t need_d = 0, need_h = 0;
        if (cudaGetLastError() != cudaSuccess ||
            cusolverDnXgeev_bufferSize(g_solver, g_params, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_NOVECTOR, n,
                                       CUDA_C_64F, dA, n, CUDA_C_64F, dW, CUDA_C_64F, nullptr, 1, CUDA_C_64F, nullptr,
                                       1, CUDA_C_64F, &need_d, &need_h) != CUSOLVER_STATUS_SUCCESS) {
            cleanup();
            return MSGPU_E_CUDA;
        }
        if (need_d > dwork_bytes) {
            cudaFree(dwork);
            dwork = nullptr;
            dwork_bytes = 0;
            if (cudaMalloc(&dwork, need_d)) {
                cleanup();
                return MSGPU_E_CUDA;
            }
            dwork_bytes = need_d;
        }
        if (need_h > hwork.size()) hwork.resize(need_h);
        if (cusolverDnXgeev(g_solver, g_params, CUSOLVER_EIG_MODE_NOVECTOR, CUSOLVER_EIG_MODE_NOVECTOR, n, CUDA_C_64F,
                            dA, n, CUDA_C_64F, dW, CUDA_C_64F, nullptr, 1, CUDA_C_64F, nullptr, 1, CUDA_C_64F, dwork,
                            dwork_bytes, hwork.empty() ? nullptr : hwork.data(), need_h,
                            dinfo) != CUSOLVER_STATUS_SUCCESS) {
            cleanup();
            return MSGPU_E_CUDA;
        }
        int info = 0;
        if (cudaMemcpy(mu + 2 * off, dW, sizeof(zc) * (size_t)n, cudaMemcpyDeviceToHost) ||
            cudaMemcpy(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost)) {
            cleanup();
            return MSGPU_E_CUDA;
        }
        // info > 0: the QR algorithm left eigenvalues unconverged (eigvals' LAPACK warning)
        if (status) status[it] = info > 0 ? MSGPU_S_NOCONV : 0;
        off += (size_t)n;
    }
    cleanup();
    return 0;
}
