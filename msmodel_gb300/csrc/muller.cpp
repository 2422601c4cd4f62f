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
// invtraceinv: every root of every realisation runs at once.  mineigval: the
// reference chains one eigenvector through every evaluation of a realisation
// -- each inverse iteration starts from the vector the previous one returned,
// root after root (ms_core.c:339-340), including the check |f(kroot)| <
// sqrt(toler) made after every search (ms_core.c:356) -- so the values of f
// depend on the order of the calls.  Here each realisation keeps its own
// vector and runs its roots one after another in the reference's order, one
// value per round, and the batch is over the realisations: every
// realisation's evaluations happen in the reference's sequence, starting from
// the constant unit vector.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>
#include "msgpu.h"
#include "error_text.h"

namespace {

using cd = std::complex<double>;

bool in_dom(const double* dom, cd z) {  // is_in_domain, src/core/domain_util.c:119 (open bounds)
    return dom[0] < z.real() && z.real() < dom[1] && dom[2] < z.imag() && z.imag() < dom[3];
}

enum Phase { START, STEP, DAMP, CHECK, CHECK0, DONE };

struct Root {
    cd z0;  // the target: kroot[i] keeps it when the search fails
    cd za, zb, zc, fa, fb, fc, zn, dz;
    double absfc = 0.0, absdz = 0.0, tol = 0.0, mu = 1.0, pow2 = 2.0;
    int s = 0;
    int nstart = 0;  // values of the start already asked for (sequential mode)
    Phase ph = START;
    bool conv = false;
};

}  // namespace

extern "C" int msgpu_find_roots_muller_batch(int method, int nmed, const msgpu_medium* media, const double* dom,
                                             int nz, const double* z0, int maxit, double toler, int precision,
                                             double* roots, int* nroots, int* nevals) {
    if ((method != MSGPU_EIG_MINEIGVAL && method != MSGPU_EIG_INVTRACEINV) || nmed < 1 || !media || !dom || nz < 0 ||
        (nz > 0 && !z0) || !roots || !nroots)
        return msg::record_error(MSGPU_E_ARG, "find_roots_muller_batch: bad argument (method mineigval or "
                                              "invtraceinv, nmed >= 1, nz >= 0, non-null pointers)");
    // find_root_muller refuses these parameters (root_finder.c:344-347): no root converges
    const bool refused = maxit <= 1 || !(toler > 0.0);
    const double DELTA = 1e-4;  // finite-difference step of root_finder.c:19
    std::vector<Root> R((size_t)nmed * nz);
    for (int m = 0; m < nmed; ++m)
        for (int i = 0; i < nz; ++i) {
            Root& r = R[(size_t)m * nz + i];
            const cd z(z0[2 * i], z0[2 * i + 1]);
            r.z0 = z;
            r.za = (1.0 - DELTA * cd(0, 1)) * z;
            r.zb = z;
            r.zc = (1.0 + DELTA * cd(0, 1)) * z;
            // refused parameters: no search, but mineigval still evaluates f at the target
            r.ph = refused ? (method == MSGPU_EIG_MINEIGVAL ? CHECK0 : DONE) : START;
        }
    const int kind = method == MSGPU_EIG_MINEIGVAL ? 4 : 3;
    const bool seq = method == MSGPU_EIG_MINEIGVAL;  // one chained eigenvector per realisation
    std::vector<int> cur(nmed, 0);                   // seq: the root of each realisation now running
    std::vector<std::vector<double>> vec(nmed);      // seq: its eigenvector, constant unit to start
    if (seq)
        for (int m = 0; m < nmed; ++m) {
            vec[m].assign(2 * (size_t)media[m].n, 0.0);
            for (int i = 0; i < media[m].n; ++i) vec[m][2 * i] = 1.0;
        }
    msgpu_job* J = nullptr;
    struct Guard {
        msgpu_job*& j;
        ~Guard() { msgpu_job_destroy(j); }
    } guard{J};
    long long ne = 0;
    std::vector<int> im;
    std::vector<double> ks, out, vin, vout;
    std::vector<int> st;
    std::vector<std::pair<size_t, int>> who;  // (root, value: 0 a, 1 b, 2 c, 3 n, 4 check, 5 check at target)
    // a search that ends without a root: for mineigval the reference still evaluates
    // f at kroot[i], which then holds the target (ms_core.c:356), and the chain of
    // eigenvectors passes through that call
    auto fail = [&](Root& r) { r.ph = seq ? CHECK0 : DONE; };
    // Muller steps of a root holding three values (root_finder.c:354-391)
    auto step = [&](Root& r) {
        const cd dfab = (r.fa - r.fb) / (r.za - r.zb), dfac = (r.fa - r.fc) / (r.za - r.zc),
                 dfbc = (r.fb - r.fc) / (r.zb - r.zc);
        const cd d1f = dfbc + dfac - dfab, d2f = (dfac - dfbc) / (r.za - r.zb);
        const cd delta = std::sqrt(d1f * d1f - 4.0 * r.fc * d2f);
        cd denom = d1f + delta;
        const cd denom1 = d1f - delta;
        if (std::abs(denom1) > std::abs(denom)) denom = denom1;
        if (denom == 0.0 || denom != denom) {  // division by zero or NaN: give up
            fail(r);
            return;
        }
        r.dz = 2.0 * r.fc / denom;
        r.absdz = std::abs(r.dz);
        r.tol = toler * std::abs(r.zc);
        if (!in_dom(dom, r.zc)) {
            fail(r);
            return;
        }
        if (r.absdz < r.tol || r.absfc == 0.0) {
            r.ph = method == MSGPU_EIG_MINEIGVAL ? CHECK : DONE;
            r.conv = method != MSGPU_EIG_MINEIGVAL;
            return;
        }
        r.mu = 1.0;
        r.pow2 = 2.0;
        r.zn = r.zc - r.mu * r.dz;
        r.ph = DAMP;
    };
    for (;;) {
        im.clear();
        ks.clear();
        who.clear();
        vin.clear();
        auto ask = [&](size_t r, int m, cd z, int w) {
            im.push_back(m);
            ks.push_back(z.real());
            ks.push_back(z.imag());
            who.emplace_back(r, w);
            if (seq) vin.insert(vin.end(), vec[m].begin(), vec[m].end());
        };
        for (int m = 0; m < nmed; ++m) {
            if (seq) {
                // the realisation's current root asks for its next value; finished roots hand on
                while (cur[m] < nz) {
                    const size_t ri = (size_t)m * nz + cur[m];
                    Root& r = R[ri];
                    if (r.ph == STEP) step(r);
                    if (r.ph == START) {
                        const cd z = r.nstart == 0 ? r.za : r.nstart == 1 ? r.zb : r.zc;
                        ask(ri, m, z, r.nstart);
                        break;
                    }
                    if (r.ph == DAMP) { ask(ri, m, r.zn, 3); break; }
                    if (r.ph == CHECK) { ask(ri, m, r.zc, 4); break; }
                    if (r.ph == CHECK0) { ask(ri, m, r.z0, 5); break; }
                    ++cur[m];  // DONE
                }
                continue;
            }
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
        }
        if (im.empty()) break;
        if (!J) {
            // capacity: one value per realisation (sequential) or every value of the first round
            const int cap = seq ? nmed : (int)im.size();
            std::vector<int> fim(cap);
            std::vector<double> fks(2 * (size_t)cap, 0.0);
            for (int i = 0; i < cap; ++i) {
                fim[i] = seq ? i : im[i];
                fks[2 * i] = seq ? 1.0 : ks[2 * i];
                fks[2 * i + 1] = seq ? 0.0 : ks[2 * i + 1];
            }
            J = msgpu_job_create(kind, nmed, media, cap, fim.data(), fks.data(), precision);
            if (!J) return MSGPU_E_CUDA;
            if (int e = msgpu_job_use_graph(J, 1)) return e;
        }
        if (int e = msgpu_job_set_points(J, (int)im.size(), im.data(), ks.data())) return e;
        if (seq)
            if (int e = msgpu_job_set_vectors(J, vin.data())) return e;
        if (int e = msgpu_job_run(J, nullptr)) return e;
        out.resize(ks.size());
        st.resize(im.size());
        if (int e = msgpu_job_results(J, out.data(), st.data())) return e;
        if (seq) {
            vout.resize(vin.size());
            if (int e = msgpu_job_amplitudes(J, vout.data())) return e;
            size_t off = 0;
            for (int m : im) {
                std::copy(vout.begin() + off, vout.begin() + off + vec[m].size(), vec[m].begin());
                off += vec[m].size();
            }
        }
        ne += (long long)im.size();
        for (size_t q = 0; q < who.size(); ++q) {
            Root& r = R[who[q].first];
            cd f(out[2 * q], out[2 * q + 1]);
            if (kind == 3) f = 1.0 / f;  // invtrinv (ms_core.c:382)
            switch (who[q].second) {
            case 0: r.fa = f; r.nstart = 1; break;
            case 1: r.fb = f; r.nstart = 2; break;
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
                if (++r.s < maxit) r.ph = STEP;
                else fail(r);
                break;
            }
            case 4:  // mineigval: the eigenvalue must be small at the root (ms_core.c:356)
                r.conv = std::abs(f) < std::sqrt(toler);
                r.ph = DONE;
                break;
            case 5:  // mineigval after a failed search: the call at the target, no root
                r.ph = DONE;
                break;
            }
        }
        if (!seq)
            for (Root& r : R)
                if (r.ph == STEP) step(r);
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
