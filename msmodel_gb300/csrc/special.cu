// special.cu -- the device special-function kernel behind msgpu_eval_special
// (engine.cu launches it): the Green functions, K_nu, F(k)^-1 and the mixed
// engine's double-float d = 3 and d = 2 elements, evaluated point by point for the
// checks against the reference goldens; a unit of its own so that it compiles
// beside the engine.
#include <cuda_runtime.h>
#include "msgpu.h"
#include "lu64.cuh"
#include "green_df.cuh"
#include "green_df2.cuh"
#include "engine_internal.h"

namespace msg {

__global__ void k_eval_special(int which, int d, msgpu_model m, int n, const double* ks, const double* rs,
                               double* out) {
    __shared__ Df3Tables tab;
    if (which >= 7) {  // block-uniform
        df3_tables_init(tab);
        __syncthreads();
    }
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    zc k = mk(ks[2 * i], ks[2 * i + 1]);
    double r = rs ? rs[i] : 1.0;
    zc v;
    switch (which) {
    case 0: v = free_green(d, k, r); break;
    case 1: v = dk_free_green(d, k, r); break;
    case 2: v = free_green_imag(d, k, r); break;
    case 3: v = bessel_k(d, k); break;
    case 5:
    case 6: {  // d = 3 matrix elements as the mixed engine evaluates them (double-float)
        dfc a, b;
        pair_elements_df3(k, r, which == 6, a, b);
        const dfc e = which == 5 ? a : b;
        v = mk(df_to_double(e.re), df_to_double(e.im));
        break;
    }
    case 7:
    case 8: {  // the same elements entirely on the FP32 pipe, as the mixed engine assembles them
        dfc a, b;
        pair_elements_df3t(tab, df_from_double(k.re), df_from_double(k.im), k.im != 0.0, df_from_double(r),
                           which == 8, a, b);
        const dfc e = which == 7 ? a : b;
        v = mk(df_to_double(e.re), df_to_double(e.im));
        break;
    }
    case 9:
    case 10: {  // d = 2 matrix elements on the FP32 pipe, as the mixed engine assembles them
        const Df2Item P = df2_item(k);
        const df rd = df_from_double(r);
        dfc a, b;
        pair_elements_df2(tab, P, rd, k_regime_df(P, rd), which == 10, a, b);
        const dfc e = which == 9 ? a : b;
        v = mk(df_to_double(e.re), df_to_double(e.im));
        break;
    }
    default: v = invf(m, d, k); break;
    }
    out[2 * i] = v.re;
    out[2 * i + 1] = v.im;
}

}  // namespace msg
