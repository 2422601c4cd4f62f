// random_function.cpp -- the random-function task of the reference
// (run_random_function_omp, src/core/ms_core.c:476-519): for every seed
// g = 0..nseed-1 (medium filled with seed g+1) and every bin i of a
// logarithmic grid of real k (get_arg_rfun, src/core/random_function_util.c:101-104)
// either the total cross section sigma(k) = -Im(phi . M^-1 phi)/k
// (total_cross_section, src/core/ms_matrix_util.c:344) or the density of
// states -Im(dlogf(k))/(2 pi k); data[g + i*nseed], every bin then sorted
// (sort_random_function, random_function_util.c:110).
//
// All nseed x nbin (medium, k) items go to the GPU as one batched job: the
// amplitude engine for the cross section, the dlogf engine for the DOS.
#include <algorithm>
#include <cmath>
#include <vector>
#include "msgpu.h"
#include "error_text.h"

extern "C" int msgpu_random_function(int type, int d, int n, int shape, double ratio, const msgpu_model* model,
                                     int nseed, int nbin, double xmin, double xmax, double* data, int* status,
                                     int precision) {
    if ((type != MSGPU_RF_CRSEC && type != MSGPU_RF_DOS) || d < 1 || n < 1 || !model || nseed < 1 || nbin < 2 ||
        !(xmin > 0.0) || !(xmax > 0.0) || !data)
        return msg::record_error(MSGPU_E_ARG, "random_function: bad argument (type crsec or dos, d, n, nseed >= 1, "
                                              "nbin >= 2, xmin and xmax > 0, non-null pointers)");
    std::vector<double> pos((size_t)nseed * n * d);
    std::vector<msgpu_medium> media(nseed);
    for (int g = 0; g < nseed; ++g) {
        double* p = pos.data() + (size_t)g * n * d;
        if (int e = msgpu_fill_medium(d, n, shape, ratio, (uint64_t)(g + 1), p)) return e;
        media[g] = msgpu_medium{d, n, p, *model};
    }
    const int nitem = nseed * nbin;
    std::vector<double> ks(2 * (size_t)nitem), out(2 * (size_t)nitem), kb(nbin);
    std::vector<int> im(nitem), st(nitem);
    for (int i = 0; i < nbin; ++i) kb[i] = xmin * std::exp(i * std::log(xmax / xmin) / (nbin - 1));
    for (int i = 0; i < nbin; ++i)
        for (int g = 0; g < nseed; ++g) {
            const int it = g + i * nseed;
            ks[2 * it] = kb[i];
            ks[2 * it + 1] = 0.0;
            im[it] = g;
        }
    int e = type == MSGPU_RF_CRSEC
                ? msgpu_amplitude_batch(nseed, media.data(), nitem, im.data(), ks.data(), out.data(), nullptr,
                                        st.data(), precision)
                : msgpu_dk_log_det_batch(nseed, media.data(), nitem, im.data(), ks.data(), out.data(), st.data(),
                                         precision);
    if (e) return e;
    for (int it = 0; it < nitem; ++it) {
        const double k = ks[2 * it];
        data[it] = type == MSGPU_RF_CRSEC ? out[2 * it] : -out[2 * it + 1] / (2 * k * 3.14159265358979323846);
        if (status) status[it] = st[it];
    }
    for (int i = 0; i < nbin; ++i) std::sort(data + (size_t)i * nseed, data + (size_t)(i + 1) * nseed);
    return 0;
}
