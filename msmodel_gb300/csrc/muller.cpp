// muller.cpp -- the root methods "mineigval" and "invtraceinv" of the
// reference's eigenstate search (find_eigenstates_serial_2 / _3,
// src/core/ms_core.c:335-401): every target runs Muller's method
// (find_root_muller, src/core/root_finder.c:342-406) on
//   mineigval   f(k) = the eigenvalue of M(k) of smallest modulus (inverse
//               iteration, ms_matrix_util.c:279), and a root counts only if
//               |f| < sqrt(toler) there (ms_core.c:356);
//   invtraceinv f(k) = 1 / tr M(k)^-1 (traceinv, ms_matrix_util.c:319).
// Then the non-converged roots are dropped and near-duplicates (relative
// 1e-14) removed, order kept (filter_cvector, uniq_cvector).
//
// Every root of every realisation is a small state machine that asks for one
// function value at a time (three at the start); each round sends all pending
// values to the GPU as one batched job (resident: set_points + run), then
// advances every machine exactly as the reference's loop would.
//
// One difference: the reference's mineigval starts each inverse iteration
// from the eigenvector of the previous call (one vector shared by all roots,
// ms_core.c:339-340); here each evaluation starts from the constant unit vector,
// as compute_eigenstates does (ms_core.c:306).  Where the iteration
// converges (|x - x_old| < 1e-10) both give the same eigenvalue.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>
#include "msgpu.h"

namespace {

using cd = std::complex<double>;

bool in_dom(const double* dom, cd z) {  // is_in_domain, src/core/domain_util.c:119 (open bounds)
    return dom[0] < z.real() && z.real() < dom[1] && dom[2] < z.imag() && z.imag() < dom[3];
}

enum Phase { START, STEP, DAMP, CHECK, DONE };

struct Root {
    cd za, zb, zc, fa, fb, fc, zn, dz;
    double absfc = 0.0, absdz = 0.0, tol = 0.0, mu = 1.0, pow2 = 2.0;
    int s = 0;
    Phase ph = START;
    bool conv = false;
};

}  // namespace

extern "C" int msgpu_find_roots_muller_batch(int method, int nmed, const msgpu_medium* media, const double* dom,
                                             int nz, const double* z0, int maxit, double toler, int precision,
                                             double* roots, int* nroots, int* nevals) {
    if ((method != MSGPU_EIG_MINEIGVAL && method != MSGPU_EIG_INVTRACEINV) || nmed < 1 || !media || !dom || nz < 0 ||
        (nz > 0 && !z0) || !roots || !nroots)
        return MSGPU_E_ARG;
    // find_root_muller refuses these parameters (root_finder.c:344-347): no root converges
    const bool refused = maxit <= 1 || !(toler > 0.0);
    const double DELTA = 1e-4;  // finite-difference step of root_finder.c:19
    std::vector<Root> R((size_t)nmed * nz);
    for (int m = 0; m < nmed; ++m)
        for (int i = 0; i < nz; ++i) {
            Root& r = R[(size_t)m * nz + i];
            const cd z(z0[2 * i], z0[2 * i + 1]);
            r.za = (1.0 - DELTA * cd(0, 1)) * z;
            r.zb = z;
            r.zc = (1.0 + DELTA * cd(0, 1)) * z;
            r.ph = refused ? DONE : START;
        }
    const int kind = method == MSGPU_EIG_MINEIGVAL ? 4 : 3;
    msgpu_job* J = nullptr;
    struct Guard {
        msgpu_job*& j;
        ~Guard() { msgpu_job_destroy(j); }
    } guard{J};
    long long ne = 0;
    std::vector<int> im;
    std::vector<double> ks, out;
    std::vector<int> st;
    std::vector<std::pair<size_t, int>> who;  // (root, which value: 0 a, 1 b, 2 c, 3 n)
    for (;;) {
        im.clear();
        ks.clear();
        who.clear();
        auto ask = [&](size_t r, int m, cd z, int w) {
            im.push_back(m);
            ks.push_back(z.real());
            ks.push_back(z.imag());
            who.emplace_back(r, w);
        };
        for (int m = 0; m < nmed; ++m)
            for (int i = 0; i < nz; ++i) {
                const size_t ri = (size_t)m * nz + i;
                Root& r = R[ri];
                if (r.ph == START) {
                    ask(ri, m, r.za, 0);
                    ask(ri, m, r.zb, 1);
                    ask(ri, m, r.zc, 2);
                } else if (r.ph == DAMP) {
                    ask(ri, m, r.zn, 3);
                } else if (r.ph == CHECK) {
                    ask(ri, m, r.zc, 4);
                }
            }
        if (im.empty()) break;
        if (!J) {
            J = msgpu_job_create(kind, nmed, media, (int)im.size(), im.data(), ks.data(), precision);
            if (!J) return MSGPU_E_CUDA;
            if (int e = msgpu_job_use_graph(J, 1)) return e;
        } else if (int e = msgpu_job_set_points(J, (int)im.size(), im.data(), ks.data())) {
            return e;
        }
        if (int e = msgpu_job_run(J, nullptr)) return e;
        out.resize(ks.size());
        st.resize(im.size());
        if (int e = msgpu_job_results(J, out.data(), st.data())) return e;
        ne += (long long)im.size();
        for (size_t q = 0; q < who.size(); ++q) {
            Root& r = R[who[q].first];
            cd f(out[2 * q], out[2 * q + 1]);
            if (kind == 3) f = 1.0 / f;  // invtrinv (ms_core.c:382)
            switch (who[q].second) {
            case 0: r.fa = f; break;
            case 1: r.fb = f; break;
            case 2: r.fc = f; r.absfc = std::abs(f); r.ph = STEP; break;
            case 3: {  // a damping sub-step (root_finder.c:392-401)
                const double absfn = std::abs(f);
                r.mu /= r.pow2;
                r.pow2 *= 2.0;
                if (absfn > r.absfc && r.mu * r.absdz > r.tol) {
                    r.zn = r.zc - r.mu * r.dz;
                    break;  // stays in DAMP: one more value
                }
                r.za = r.zb; r.fa = r.fb;
                r.zb = r.zc; r.fb = r.fc;
                r.zc = r.zn; r.fc = f; r.absfc = absfn;
                r.ph = ++r.s < maxit ? STEP : DONE;
                break;
            }
            case 4:  // mineigval: the eigenvalue must be small at the root (ms_core.c:356)
                r.conv = std::abs(f) < std::sqrt(toler);
                r.ph = DONE;
                break;
            }
        }
        // Muller steps of every root now holding three values (root_finder.c:354-391)
        for (Root& r : R) {
            if (r.ph != STEP) continue;
            const cd dfab = (r.fa - r.fb) / (r.za - r.zb), dfac = (r.fa - r.fc) / (r.za - r.zc),
                     dfbc = (r.fb - r.fc) / (r.zb - r.zc);
            const cd d1f = dfbc + dfac - dfab, d2f = (dfac - dfbc) / (r.za - r.zb);
            const cd delta = std::sqrt(d1f * d1f - 4.0 * r.fc * d2f);
            cd denom = d1f + delta;
            const cd denom1 = d1f - delta;
            if (std::abs(denom1) > std::abs(denom)) denom = denom1;
            if (denom == 0.0 || denom != denom) {  // division by zero or NaN: give up
                r.ph = DONE;
                continue;
            }
            r.dz = 2.0 * r.fc / denom;
            r.absdz = std::abs(r.dz);
            r.tol = toler * std::abs(r.zc);
            if (!in_dom(dom, r.zc)) {
                r.ph = DONE;
                continue;
            }
            if (r.absdz < r.tol || r.absfc == 0.0) {
                r.ph = method == MSGPU_EIG_MINEIGVAL ? CHECK : DONE;
                r.conv = method != MSGPU_EIG_MINEIGVAL;
                continue;
            }
            r.mu = 1.0;
            r.pow2 = 2.0;
            r.zn = r.zc - r.mu * r.dz;
            r.ph = DAMP;
        }
    }
    // filter_cvector then uniq_cvector (relative 1e-14), order kept
    for (int m = 0; m < nmed; ++m) {
        std::vector<cd> ok;
        for (int i = 0; i < nz; ++i) {
            const Root& r = R[(size_t)m * nz + i];
            if (!r.conv) continue;
            bool uniq = true;
            for (const cd& u : ok)
                if (std::abs(r.zc - u) < 1e-14 * std::abs(r.zc) || std::abs(r.zc - u) < 1e-14) {
                    uniq = false;
                    break;
                }
            if (uniq) ok.push_back(r.zc);
        }
        nroots[m] = (int)ok.size();
        for (size_t i = 0; i < ok.size(); ++i) {
            roots[2 * ((size_t)m * nz + i)] = ok[i].real();
            roots[2 * ((size_t)m * nz + i) + 1] = ok[i].imag();
        }
    }
    if (nevals) *nevals = (int)std::min<long long>(ne, 2147483647LL);
    return 0;
}
