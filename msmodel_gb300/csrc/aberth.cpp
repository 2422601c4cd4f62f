// aberth.cpp -- batched resonance search: the Maehly-Aberth-Ehrlich iteration
// of the reference (solve_aberth, src/core/root_finder.c:522-577, driven by
// find_eigenstates_serial_1, src/core/ms_core.c:320-328) over many
// realisations at once.
//
// In the reference's Gauss-Seidel sweep, root i's dlogf is evaluated at z_i
// before z_i moves in that sweep, so the dlogf values of all roots still in
// progress can be computed together at the start of the sweep -- one batched
// GPU job over every (realisation, root) -- and the sweep then replays the
// reference's sequential update exactly: the repulsion sum sees the roots
// j < i already moved.  The updates, flags and the background polynomial
// (least squares on 6*nexpsup Halton samples, root_finder.c:161) are FP64 on
// the host; all dlogf evaluations are on the GPU.
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

// Least squares min |A x - b| for A (m x nc, column-major) by Householder QR;
// the reference calls zgels_ (root_finder.c:59-68).  x returned in b[0..nc).
void least_squares(int m, int nc, std::vector<cd>& a, std::vector<cd>& b) {
    for (int j = 0; j < nc; ++j) {
        double nrm = 0.0;
        for (int i = j; i < m; ++i) nrm += std::norm(a[i + j * m]);
        nrm = std::sqrt(nrm);
        if (nrm == 0.0) continue;
        cd x0 = a[j + j * m];
        cd alpha = (std::abs(x0) > 0 ? -x0 / std::abs(x0) : cd(-1.0)) * nrm;
        a[j + j * m] -= alpha;
        double vn = 0.0;
        for (int i = j; i < m; ++i) vn += std::norm(a[i + j * m]);
        for (int c = j + 1; c < nc; ++c) {
            cd s = 0.0;
            for (int i = j; i < m; ++i) s += std::conj(a[i + j * m]) * a[i + c * m];
            s = 2.0 * s / vn;
            for (int i = j; i < m; ++i) a[i + c * m] -= s * a[i + j * m];
        }
        cd s = 0.0;
        for (int i = j; i < m; ++i) s += std::conj(a[i + j * m]) * b[i];
        s = 2.0 * s / vn;
        for (int i = j; i < m; ++i) b[i] -= s * a[i + j * m];
        a[j + j * m] = alpha;
    }
    for (int j = nc - 1; j >= 0; --j) {
        cd s = b[j];
        for (int c = j + 1; c < nc; ++c) s -= a[j + c * m] * b[c];
        b[j] = s / a[j + j * m];
    }
}

struct Realisation {
    std::vector<cd> z;
    std::vector<int> flag;  // 0 in progress, 1 converged, -1 failed, 2 parked (mixed: FP64 finish pending)
    std::vector<int> used;  // sweeps this root has taken part in
    std::vector<cd> poly;
    int nr = 0;
    bool aborted = false;
};

}  // namespace

extern "C" int msgpu_solve_aberth_batch(int nmed, const msgpu_medium* media, const double* dom, int nz,
                                        const double* z0, int nexpsup, int maxit, double toler, int precision,
                                        double* roots, int* nroots, int* nevals) {
    if (nmed < 1 || !media || !dom || nz < 0 || (nz > 0 && !z0) || nexpsup < 0 || nexpsup > 16 || maxit < 0 ||
        !roots || !nroots)
        return msg::record_error(MSGPU_E_ARG, "solve_aberth_batch: bad argument (nmed >= 1, nz >= 0, nexpsup in "
                                              "0..16, maxit >= 0, non-null pointers)");
    std::vector<Realisation> R(nmed);
    long long ne = 0;
    for (int r = 0; r < nmed; ++r) {
        std::vector<cd>& z = R[r].z;
        for (int i = 0; i < nz; ++i) z.emplace_back(z0[2 * i], z0[2 * i + 1]);
        // uniq_cvector (complex_vector_util.c:130): drop near-duplicates, keep order
        int size = z.empty() ? 0 : 1;
        for (int i = 1; i < (int)z.size(); ++i) {
            bool uniq = true;
            for (int j = 0; j < size; ++j)
                if (std::abs(z[i] - z[j]) < toler * std::abs(z[i]) || std::abs(z[i] - z[j]) < toler) {
                    uniq = false;
                    break;
                }
            if (uniq) {
                std::swap(z[i], z[size]);
                ++size;
            }
        }
        z.resize(size);
        // exclude_from_domain (domain_util.c:133), order kept
        std::vector<cd> kept;
        for (cd v : z)
            if (in_dom(dom, v)) kept.push_back(v);
        z = kept;
        R[r].nr = (int)z.size();
        R[r].flag.assign(z.size(), 0);
        // fewer than two starting points: the reference gives up (root_finder.c:525-528)
        R[r].aborted = R[r].nr <= 1;
    }
    const int deg = nexpsup - 1;
    // One resident dlogf job per precision serves every evaluation of the
    // search: the media are uploaded once, each batch replaces the points and
    // replays the captured run.
    struct Jobs {
        msgpu_job* j[2] = {nullptr, nullptr};
        ~Jobs() {
            msgpu_job_destroy(j[0]);
            msgpu_job_destroy(j[1]);
        }
    } jobs;
    const int cap = nmed * std::max(std::max(nz, 6 * nexpsup), 1);
    auto dlogf_batch = [&](int prec, const std::vector<int>& im, const std::vector<double>& ks, std::vector<double>& out,
                           std::vector<int>& st) -> int {
        msgpu_job*& J = jobs.j[prec == MSGPU_MIXED ? 1 : 0];
        if (!J) {
            std::vector<int> fim(cap);
            std::vector<double> fks(2 * (size_t)cap, 0.0);
            for (int i = 0; i < cap; ++i) {
                fim[i] = i % nmed;
                fks[2 * i] = 1.0;
            }
            J = msgpu_job_create(1, nmed, media, cap, fim.data(), fks.data(), prec);
            if (!J) return MSGPU_E_CUDA;
            if (int e = msgpu_job_use_graph(J, 1)) return e;
        }
        if (int e = msgpu_job_set_points(J, (int)im.size(), im.data(), ks.data())) return e;
        if (int e = msgpu_job_run(J, nullptr)) return e;
        return msgpu_job_results(J, out.data(), st.data());
    };
    if (nexpsup > 0) {
        const int ns = 6 * nexpsup;
        std::vector<double> hz(2 * ns);
        msgpu_halton_points(dom, ns, hz.data());
        std::vector<int> im;
        std::vector<double> ks;
        for (int r = 0; r < nmed; ++r) {
            if (R[r].aborted) continue;
            for (int i = 0; i < ns; ++i) {
                im.push_back(r);
                ks.push_back(hz[2 * i]);
                ks.push_back(hz[2 * i + 1]);
            }
        }
        if (!im.empty()) {
            std::vector<double> out(ks.size());
            std::vector<int> st(im.size());
            int e = dlogf_batch(precision, im, ks, out, st);
            if (e) return e;
            ne += (long long)im.size();
            size_t q = 0;
            for (int r = 0; r < nmed; ++r) {
                if (R[r].aborted) continue;
                std::vector<cd> a((size_t)ns * nexpsup), b(ns);
                for (int i = 0; i < ns; ++i, ++q) {
                    cd zi(hz[2 * i], hz[2 * i + 1]), zp = 1.0;
                    for (int j = 0; j < nexpsup; ++j) {
                        a[i + j * ns] = zp;
                        zp *= zi;
                    }
                    b[i] = cd(out[2 * q], out[2 * q + 1]);
                }
                least_squares(ns, nexpsup, a, b);
                R[r].poly.assign(b.begin(), b.begin() + nexpsup);
            }
        }
    }
    // Mixed precision.  Near a root M is nearly singular and tr(M^-1 dM/dk)
    // magnifies the factorisation's error by its condition number, so a root
    // whose relative step falls below SWITCH in mixed precision is parked (the
    // step applied) and later finished with FP64 dlogf.  A mixed step that
    // already meets the reference's stop test |dz| < toler |z| ends the root
    // as in the reference (the mixed dlogf is sliced six ways, ~1e-11
    // relative, so the test decides as FP64 would).  Every root keeps the
    // reference's budget of maxit sweeps in all (root_finder.c:545-576): the
    // FP64 sweeps of a parked root count against the sweeps it has used, and
    // a root still in progress when its budget is spent fails.  The
    // Newton/Aberth update is FP64 throughout.
    constexpr double SWITCH = 1e-9;
    // One sweep over every realisation: batched dlogf of the roots in progress
    // (flag 0) at precision prec, then the reference's sequential update.
    // Returns false when no root is in progress or on a GPU error.
    auto sweep = [&](int prec, int& err) -> bool {
        std::vector<int> im;
        std::vector<double> ks;
        for (int r = 0; r < nmed; ++r) {
            if (R[r].aborted) continue;
            for (int i = 0; i < R[r].nr; ++i)
                if (R[r].flag[i] == 0) {
                    im.push_back(r);
                    ks.push_back(R[r].z[i].real());
                    ks.push_back(R[r].z[i].imag());
                }
        }
        if (im.empty()) return false;
        std::vector<double> out(ks.size());
        std::vector<int> st(im.size());
        err = dlogf_batch(prec, im, ks, out, st);
        if (err) return false;
        ne += (long long)im.size();
        size_t q = 0;
        for (int r = 0; r < nmed; ++r) {
            if (R[r].aborted) continue;
            Realisation& X = R[r];
            for (int i = 0; i < X.nr; ++i) {
                if (X.flag[i] != 0) continue;
                ++X.used[i];
                cd pv = 0.0;
                if (deg >= 0) {
                    pv = X.poly[deg];
                    for (int j = deg - 1; j >= 0; --j) pv = pv * X.z[i] + X.poly[j];
                }
                cd inv = cd(out[2 * q], out[2 * q + 1]) - pv;
                ++q;
                for (int j = 0; j < X.nr; ++j)
                    if (j != i) inv -= 1.0 / (X.z[i] - X.z[j]);
                cd dz = 1.0 / inv, zn = X.z[i] - dz;
                if (!in_dom(dom, zn)) {
                    X.flag[i] = -1;
                } else if (std::abs(dz) < toler * std::abs(X.z[i])) {
                    X.flag[i] = 1;
                } else {
                    if (prec == MSGPU_MIXED && std::abs(dz) < SWITCH * std::abs(X.z[i])) X.flag[i] = 2;  // parked
                    X.z[i] = zn;
                }
            }
        }
        return true;
    };
    for (int r = 0; r < nmed; ++r) R[r].used.assign(R[r].nr, 0);
    int err = 0;
    for (int s = 0; s < maxit && sweep(precision, err); ++s) {
    }
    if (err) return err;
    if (precision == MSGPU_MIXED) {
        // FP64 finish of the parked roots, each within its remaining budget
        for (int r = 0; r < nmed; ++r)
            for (int i = 0; i < R[r].nr; ++i)
                if (R[r].flag[i] == 2) R[r].flag[i] = 0;
                else if (R[r].flag[i] == 0) R[r].flag[i] = -1;  // budget spent in mixed precision
        for (;;) {
            for (int r = 0; r < nmed; ++r)
                for (int i = 0; i < R[r].nr; ++i)
                    if (R[r].flag[i] == 0 && R[r].used[i] >= maxit) R[r].flag[i] = -1;
            if (!sweep(MSGPU_FP64, err)) break;
        }
        if (err) return err;
    }
    for (int r = 0; r < nmed; ++r) {
        Realisation& X = R[r];
        std::vector<cd> ok;
        if (X.aborted) {
            ok = X.z;
        } else {
            for (int i = 0; i < X.nr; ++i)
                if (X.flag[i] == 1) ok.push_back(X.z[i]);
            std::stable_sort(ok.begin(), ok.end(), [](cd a, cd b) { return a.real() < b.real(); });
        }
        nroots[r] = (int)ok.size();
        for (size_t i = 0; i < ok.size(); ++i) {
            roots[2 * ((size_t)r * nz + i)] = ok[i].real();
            roots[2 * ((size_t)r * nz + i) + 1] = ok[i].imag();
        }
    }
    if (nevals) *nevals = (int)std::min<long long>(ne, 2147483647LL);
    return 0;
}
