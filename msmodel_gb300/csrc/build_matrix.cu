// build_matrix.cu -- the single-matrix assembly kernel behind the drop-in
// build_ms_matrix / build_dk_ms_matrix (engine.cu launches it); a unit of its
// own so that it compiles beside the engine instead of after it.
#include <cuda_runtime.h>
#include "msgpu.h"
#include "lu64.cuh"
#include "green_df.cuh"
#include "engine_internal.h"

namespace msg {

// single-matrix kernels used by the drop-in layer ---------------------------------
__global__ void __launch_bounds__(NT, 1) k_build_matrix(zc* A, int n, int d, const double* pos, msgpu_model m,
                                                        double kre, double kim, int deriv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LuSmem& s = *reinterpret_cast<LuSmem*>(smem_raw);
    // a grid of CTAs shares the column tiles: CTA b assembles column tiles J = b, b + grid, ...
    const int tid = threadIdx.x;
    const zc k = mk(kre, kim);
    if (tid == 0) s.diag[0] = deriv ? dk_invf(m, d, k) : invf(m, d, k);
    __syncthreads();
    const int nt = (n + 31) / 32;
    for (int J = blockIdx.x; J < nt; J += gridDim.x) {
        for (int I = 0; I <= J; ++I) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int ii = tid & 31, jj = (tid >> 5) + 8 * q;
                const int i = I * 32 + ii, j = J * 32 + jj;
                if (i < n && j < n && i <= j) {
                    zc v;
                    if (i < j) {
                        zc mm, dm;
                        pair_elements(d, k, atom_distance(d, pos, i, j), deriv != 0, mm, dm);
                        v = deriv ? dm : mm;
                    } else {
                        v = s.diag[0];
                    }
                    A[i + (size_t)j * n] = v;
                    s.T[jj][ii] = v;
                }
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int jj = tid & 31, ii = (tid >> 5) + 8 * q;
                const int i = I * 32 + ii, j = J * 32 + jj;
                if (j < n && i < j) A[j + (size_t)i * n] = s.T[jj][ii];
            }
            __syncthreads();
        }
    }
}

}  // namespace msg
