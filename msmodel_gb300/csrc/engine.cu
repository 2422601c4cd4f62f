// engine.cu -- batched Foldy-Lax engine: persistent kernels over a device
// work queue, the runtime (device, workspace, jobs) and the msgpu_* C ABI.
//
// One CTA takes the next (k, realisation) item from an atomic counter,
// assembles M(k) (and dM/dk) into its private slot of the workspace, factors
// it and reduces the trace-log or the trace of M^-1 dM/dk, then takes the
// next item.  Items are dealt largest-n first, so uneven sizes balance.
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "msgpu.h"
#include "lu64.cuh"
#include "green_df.cuh"
#include "engine_internal.h"

using namespace msg;

namespace msg {

// complex elements of one CTA slot: the matrix, plus dM/dk (kind 1) or the
// right-hand side (kind 2)
__host__ __device__ inline size_t slot_elems(int kind, size_t slot, int nmax) {
    if (kind == 1) return 2 * slot;
    // kind 2: the matrix, its copy for the refinement residual (mixed engine), four vectors;
    // kinds 1, 3: the matrix and a right-hand-side matrix; kind 4: the matrix and two vectors
    const size_t vec = (((size_t)nmax + 15) / 16) * 16;
    if (kind == 2) return 2 * slot + 4 * vec;
    if (kind == 1 || kind == 3) return 2 * slot;
    if (kind == 4) return slot + 2 * vec;
    return slot;
}

// cnormalize (complex_vector_util.c:47): x /= fac, fac = |x| x_i0/|x_i0| with
// x_i0 the first nonzero entry (locks the phase); returns fac
static __device__ zc cnormalize_block(zc* __restrict__ x, int n, LuSmem& s) {
    double nr = 0.0, z0 = 0.0, z1 = 0.0;
    for (int i = threadIdx.x; i < n; i += NT) nr += zabs2(x[i]);
    block_sum3(nr, z0, z1, s);
    double nzv = -1.0;
    int nzi = n;
    for (int i = threadIdx.x; i < n; i += NT)
        if (x[i].re != 0.0 || x[i].im != 0.0) {
            nzv = 1.0;
            nzi = min(nzi, i);
        }
    int i0;
    block_argmax(nzv, nzi, s, i0);
    if (i0 >= n) return mk(1.0);
    const zc xi = x[i0];
    const zc fac = (sqrt(nr) / zabs(xi)) * xi;
    __syncthreads();  // every thread read x[i0] before it is rescaled
    const zc rf = 1.0 / fac;
    for (int i = threadIdx.x; i < n; i += NT) x[i] = x[i] * rf;
    __syncthreads();
    return fac;
}

// inverse_iteration (ms_matrix_util.c:279) on the LU already in A: from
// `start` (n complex values, the caller's previous eigenvector) or else the
// constant unit vector, x <- normalize(A^-1 x) until |x - x_old| < 1e-10 or 50
// steps (the reference's ivit_maxit / ivit_toler); returns lambda = 1 / fac,
// the eigenvalue of smallest modulus, x the eigenvector; conv = 0 if not reached.
static __device__ zc inverse_iteration(const zc* __restrict__ A, zc* __restrict__ x, zc* __restrict__ xold, int n,
                                       const int* __restrict__ ipiv, LuSmem& s, int& conv,
                                       const double* __restrict__ start) {
    for (int i = threadIdx.x; i < n; i += NT) x[i] = start ? mk(start[2 * i], start[2 * i + 1]) : mk(1.0);
    __syncthreads();
    zc fac = cnormalize_block(x, n, s);
    conv = 0;
    for (int it = 0; it < 50; ++it) {
        for (int i = threadIdx.x; i < n; i += NT) xold[i] = x[i];
        __syncthreads();
        lu_solve_vec(A, x, n, ipiv, s);
        fac = cnormalize_block(x, n, s);
        double d2 = 0.0, z0 = 0.0, z1 = 0.0;
        for (int i = threadIdx.x; i < n; i += NT) d2 += zabs2(x[i] - xold[i]);
        block_sum3(d2, z0, z1, s);
        if (sqrt(d2) < 1e-10) {
            conv = 1;
            break;
        }
    }
    return 1.0 / fac;
}

__global__ void __launch_bounds__(NT, 2) k_engine_fp64(EngineParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LuSmem& s = *reinterpret_cast<LuSmem*>(smem_raw);
    zc* A = P.ws + (size_t)blockIdx.x * slot_elems(P.kind, P.slot, P.piv_stride);
    zc* B = (P.kind >= 1) ? A + P.slot : nullptr;
    int* ipiv = P.piv + (size_t)blockIdx.x * P.piv_stride;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned q = atomicAdd(P.counter, 1u);
            s.item = q < P.counter[1] ? (int)q : P.nitem;
            s.info = 0;
        }
        __syncthreads();
        const int q = s.item;
        if (q >= P.nitem) break;
        const int it = P.order[q];
        const MedDev md = P.media[P.item_med[it]];
        const zc k = mk(P.ks[2 * it], P.ks[2 * it + 1]);
        assemble(A, P.kind == 1 ? B : nullptr, md.n, md.d, md.pos, md.model, k, s);
        zc res;
        int conv = 1;
        if (P.kind == 3) {
            // traceinv (ms_matrix_util.c:319): tr(M^-1 I) by the n-right-hand-side solve
            for (size_t e = threadIdx.x; e < (size_t)md.n * md.n; e += NT)
                B[e] = (e % (md.n + 1) == 0) ? mk(1.0) : mk(0.0);
            __syncthreads();
        }
        if (P.kind == 2) {
            // incident plane wave along +x (reference incident_wave_util.c:76, ms_core.c:616-618)
            for (int i = threadIdx.x; i < md.n; i += NT) B[i] = zexp(mk(0.0, 1.0) * k * md.pos[i * md.d]);
            __syncthreads();
        }
        lu_factor(A, md.n, ipiv, s);
        if (P.kind == 0) {
            res = lu_tracelog(A, md.n, ipiv, s);
        } else if (P.kind == 1 || P.kind == 3) {
            res = lu_trace_solve(A, B, md.n, ipiv, s);
        } else if (P.kind == 4) {
            const size_t vec = (((size_t)P.piv_stride + 15) / 16) * 16;
            res = inverse_iteration(A, B, B + vec, md.n, ipiv, s, conv,
                                    P.warm && P.amps ? P.amps + 2 * P.amp_off[it] : nullptr);
            if (P.amps)
                for (int i = threadIdx.x; i < md.n; i += NT) {
                    P.amps[2 * (P.amp_off[it] + i)] = B[i].re;
                    P.amps[2 * (P.amp_off[it] + i) + 1] = B[i].im;
                }
        } else {
            lu_solve_vec(A, B, md.n, ipiv, s);
            // optical theorem sigma = -Im(conj(phi).a)/k (reference ms_matrix_util.c:361)
            double dr = 0.0, di = 0.0, z = 0.0;
            for (int i = threadIdx.x; i < md.n; i += NT) {
                zc ph = zexp(mk(0.0, 1.0) * k * md.pos[i * md.d]);
                zc t = conjz(ph) * B[i];
                dr += t.re;
                di += t.im;
                if (P.amps) {
                    P.amps[2 * (P.amp_off[it] + i)] = B[i].re;
                    P.amps[2 * (P.amp_off[it] + i) + 1] = B[i].im;
                }
            }
            block_sum3(dr, di, z, s);
            res = mk(-di, 0.0) / k;
        }
        if (threadIdx.x == 0) {
            P.out[2 * it] = res.re;
            P.out[2 * it + 1] = res.im;
            int st = 0;
            if (s.info) st |= MSGPU_S_SINGULAR;
            if (!isfinite(res.re) || !isfinite(res.im)) st |= MSGPU_S_NONFINITE;
            if (!conv) st |= MSGPU_S_NOCONV;
            P.status[it] = st;
        }
        __syncthreads();
    }
}

// single-matrix assembly for the drop-in layer (build_matrix.cu)
__global__ void __launch_bounds__(NT, 1) k_build_matrix(zc* A, int n, int d, const double* pos, msgpu_model m,
                                                        double kre, double kim, int deriv);

__global__ void __launch_bounds__(NT, 1) k_tracelog_matrix(zc* A, int n, int* ipiv, double* out, int* info) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    LuSmem& s = *reinterpret_cast<LuSmem*>(smem_raw);
    if (threadIdx.x == 0) s.info = 0;
    __syncthreads();
    lu_factor(A, n, ipiv, s);
    zc r = lu_tracelog(A, n, ipiv, s);
    if (threadIdx.x == 0) {
        out[0] = r.re;
        out[1] = r.im;
        *info = s.info;
    }
}

// device special functions for the checks against the reference goldens (special.cu)
__global__ void k_eval_special(int which, int d, msgpu_model m, int n, const double* ks, const double* rs,
                               double* out);

// FP64 FMA throughput probe: 8 independent chains per thread; the roofline
// denominator of the plain (FP64-pipe-bound) path.
__global__ void k_probe_dfma(double* sink, int iters, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
           x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) sink[blockIdx.x] = s;
}

// FP64 tensor-core throughput probe: 8 independent accumulators per warp of the
// warp-level m8n8k4 FP64 MMA (512 flops each), the other candidate of the FP64 path
__global__ void k_probe_dmma(double* sink, int iters, double a, double b) {
    double c[8][2];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        c[u][0] = threadIdx.x + u;
        c[u][1] = 0.5 * u;
    }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(c[u][0]), "+d"(c[u][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int u = 0; u < 8; ++u) s += c[u][0] + c[u][1];
    if (s == 12345.678) sink[blockIdx.x] = s;
}

}  // namespace msg

// ---------------------------------------------------------------------------
// runtime
// ---------------------------------------------------------------------------
namespace {

std::mutex g_mu;
std::string g_err;
int g_dev = -1;
int g_sms = 0;
int g_ctas_fp64 = 0;
std::atomic<uint64_t> g_launches{0};
void* g_ws = nullptr;
size_t g_ws_bytes = 0;
unsigned long long g_ws_gen = 1;  // changes whenever g_ws moves (captured graphs hold its address)

// Launch choices per (kind, requested precision, size bucket): the engine that
// runs (a mixed request may be served by the FP64 engine, which is at least as
// accurate) and the resident CTAs per SM of the persistent grid.  0 = default
// (the requested engine, as many CTAs as fit).  Filled by msgpu_autotune or
// msgpu_tune_set; bucket b holds nmax in (2^(b-1), 2^b].
struct TuneEntry {
    int engine = 0;  // 0 default, 1 + MSGPU_FP64 / 1 + MSGPU_MIXED
    int ctas = 0;
};
constexpr int TUNE_BUCKETS = 17;
TuneEntry g_tune[3][2][TUNE_BUCKETS];

int size_bucket(int n) {
    int b = 0;
    while ((1 << b) < n && b < TUNE_BUCKETS - 1) ++b;
    return b;
}

int set_err(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return set_err(MSGPU_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t smem_bytes() { return sizeof(LuSmem); }

int init_locked(int device) {
    if (g_dev >= 0) return 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_err(MSGPU_E_NODEV, "no CUDA device");
    if (device < 0) device = 0;
    CK(cudaSetDevice(device));
    cudaDeviceProp pr;
    CK(cudaGetDeviceProperties(&pr, device));
    g_sms = pr.multiProcessorCount;
    CK(cudaFuncSetAttribute(k_engine_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes()));
    CK(cudaFuncSetAttribute(k_build_matrix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes()));
    CK(cudaFuncSetAttribute(k_tracelog_matrix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes()));
    int occ = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_engine_fp64, NT, smem_bytes()));
    g_ctas_fp64 = std::max(1, occ);
    g_dev = device;
    return 0;
}

int ensure_ws(size_t bytes, void** p) {
    if (bytes > g_ws_bytes) {
        if (g_ws) cudaFree(g_ws);
        g_ws = nullptr;
        g_ws_bytes = 0;
        ++g_ws_gen;
        CK(cudaMalloc(&g_ws, bytes));
        g_ws_bytes = bytes;
    }
    *p = g_ws;
    return 0;
}

}  // namespace

// workspace budget for the per-CTA matrix slots
static size_t ws_budget() {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    size_t cap = (size_t)160 << 30;
    size_t avail = fr + g_ws_bytes;
    return std::min(cap, avail > ((size_t)4 << 30) ? avail - ((size_t)4 << 30) : avail / 2);
}

struct msgpu_job {
    int kind = 0, precision = 0, nitem = 0, nmed = 0, nmax = 0;
    int cap = 0;  // item capacity of the device arrays
    double flops = 0.0;
    int grid = 0;
    std::vector<int> med_n;  // n of every medium (host copy)
    // mixed engine: per medium the smallest and largest pair distance (d = 3 with the
    // "maximum" model), or a negative smallest distance where the entry span is not predicted
    std::vector<double> med_rmin, med_rmax;
    bool wide = false;       // some item may need six-way slicing (sticky: captured graphs keep it)
    bool warm = false;       // kind 4: inverse iterations start from the vectors set by msgpu_job_set_vectors
    bool d3only = true;      // every medium has d = 3
    MedDev* d_media = nullptr;
    double* d_pos = nullptr;
    double* d_ks = nullptr;
    int* d_item_med = nullptr;
    int* d_order = nullptr;
    double* d_out = nullptr;
    int* d_status = nullptr;
    unsigned* d_counter = nullptr;  // [0] work queue, [1] live items
    int* d_piv = nullptr;
    size_t slot = 0;
    size_t ws_bytes = 0;
    long long amp_total = 0, amp_cap = 0;
    double* d_amps = nullptr;
    long long* d_amp_off = nullptr;
    // graph mode: the run (queue reset + engine launch) captured once and replayed
    bool use_graph = false;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    unsigned long long gen = 0;
};

extern "C" {

}  // extern "C"

namespace msg {
void count_launches(int n) { g_launches += n; }
// for entry points outside this file's lock (the allocation-free and eigenvalue entries)
int record_error(int code, const char* what) {
    std::lock_guard<std::mutex> lk(g_mu);
    return set_err(code, what);
}
}  // namespace msg

extern "C" {

int msgpu_init(int device) {
    std::lock_guard<std::mutex> lk(g_mu);
    return init_locked(device);
}

const char* msgpu_last_error(void) { return g_err.c_str(); }

int msgpu_sm_count(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (init_locked(-1)) return 0;
    return g_sms;
}

uint64_t msgpu_launch_count(void) { return g_launches.load(); }

int msgpu_probe_fp64(double* tflops) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (int e = init_locked(-1)) return e;
    double* sink = nullptr;
    CK(cudaMalloc(&sink, sizeof(double) * 4096));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int blocks = g_sms * 4, threads = 256, iters = 8192;
    k_probe_dfma<<<blocks, threads>>>(sink, 64, 0.999999, 1e-7);  // warm-up
    g_launches++;
    CK(cudaEventRecord(e0));
    k_probe_dfma<<<blocks, threads>>>(sink, iters, 0.999999, 1e-7);
    g_launches++;
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return 0;
}

int msgpu_probe_fp64_mma(double* tflops) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (int e = init_locked(-1)) return e;
    double* sink = nullptr;
    CK(cudaMalloc(&sink, sizeof(double) * 4096));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int blocks = g_sms * 4, threads = 256, iters = 2048;
    k_probe_dmma<<<blocks, threads>>>(sink, 16, 0.999999, 1e-7);  // warm-up
    g_launches++;
    CK(cudaEventRecord(e0));
    k_probe_dmma<<<blocks, threads>>>(sink, iters, 0.999999, 1e-7);
    g_launches++;
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    // 512 flops per warp-level MMA, 8 per warp and iteration
    *tflops = 512.0 * 8.0 * iters * (double)blocks * (threads / 32) / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return 0;
}

int msgpu_eval_special(int which, int d, const msgpu_model* model, int n, const double* ks, const double* rs,
                       double* out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (int e = init_locked(-1)) return e;
    if (n <= 0) return 0;
    msgpu_model m{};
    if (model) m = *model;
    double *dk = nullptr, *dr = nullptr, *dout = nullptr;
    CK(cudaMalloc(&dk, sizeof(double) * 2 * n));
    CK(cudaMalloc(&dout, sizeof(double) * 2 * n));
    if (rs) CK(cudaMalloc(&dr, sizeof(double) * n));
    CK(cudaMemcpy(dk, ks, sizeof(double) * 2 * n, cudaMemcpyHostToDevice));
    if (rs) CK(cudaMemcpy(dr, rs, sizeof(double) * n, cudaMemcpyHostToDevice));
    k_eval_special<<<(n + 127) / 128, 128>>>(which, d, m, n, dk, dr, dout);
    g_launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpy(out, dout, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    cudaFree(dk);
    cudaFree(dout);
    if (dr) cudaFree(dr);
    return 0;
}

int msgpu_build_matrix(const msgpu_medium* med, const double* k, int deriv, double* mat) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (int e = init_locked(-1)) return e;
    if (!med || med->n < 1 || med->d < 1 || !med->pos || !k || !mat) return set_err(MSGPU_E_ARG, "bad argument");
    const int n = med->n, d = med->d;
    double* dpos = nullptr;
    zc* dA = nullptr;
    CK(cudaMalloc(&dpos, sizeof(double) * (size_t)n * d));
    CK(cudaMalloc(&dA, sizeof(zc) * (size_t)n * n));
    CK(cudaMemcpy(dpos, med->pos, sizeof(double) * (size_t)n * d, cudaMemcpyHostToDevice));
    int nt = (n + 31) / 32;
    k_build_matrix<<<std::min(nt, 4 * g_sms), NT, smem_bytes()>>>(dA, n, d, dpos, med->model, k[0], k[1], deriv);
    g_launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpy(mat, dA, sizeof(zc) * (size_t)n * n, cudaMemcpyDeviceToHost));
    cudaFree(dpos);
    cudaFree(dA);
    return 0;
}

int msgpu_tracelog_matrix(int n, const double* mat, double* out, int* info) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (int e = init_locked(-1)) return e;
    if (n < 1 || !mat || !out) return set_err(MSGPU_E_ARG, "bad argument");
    zc* dA = nullptr;
    int* dp = nullptr;
    double* dout = nullptr;
    CK(cudaMalloc(&dA, sizeof(zc) * (size_t)n * n));
    CK(cudaMalloc(&dp, sizeof(int) * (size_t)n + 64));
    CK(cudaMalloc(&dout, 64));
    CK(cudaMemcpy(dA, mat, sizeof(zc) * (size_t)n * n, cudaMemcpyHostToDevice));
    k_tracelog_matrix<<<1, NT, smem_bytes()>>>(dA, n, dp, dout, reinterpret_cast<int*>(dout + 2));
    g_launches++;
    CK(cudaGetLastError());
    double h[3];
    CK(cudaMemcpy(h, dout, sizeof(double) * 3, cudaMemcpyDeviceToHost));
    out[0] = h[0];
    out[1] = h[1];
    if (info) std::memcpy(info, &h[2], sizeof(int));
    cudaFree(dA);
    cudaFree(dp);
    cudaFree(dout);
    return 0;
}

// Could the entries of M(k) (and of dM/dk for kind 1) of an item span more
// than the mixed engine's four-slice budget?  For d = 3 and the "maximum"
// model the moduli are known in closed form: off the diagonal
// |G| = e^{a r} / (4 pi r) (a = -Im k) and |dG/dk| = e^{a r} / (4 pi) over the
// pair distances [rmin, rmax], on the diagonal |k| / (4 pi) and 1 / (4 pi).
// The predicted span of the moduli, times 2 sqrt 2 (the engine measures
// max(|Re|, |Im|), within sqrt 2 of the modulus), is compared with the
// engine's threshold for the job kind; anything not covered counts as wide.
static bool item_may_be_wide(double rmin, double rmax, int kind, double kre, double kim) {
    // the engine's thresholds: 2^8, or 2^20 for amplitude items (refined to an FP64 residual)
    const double thr = kind == 2 ? 1048576.0 : 256.0;
    if (!(rmin > 0.0) || !(rmax >= rmin)) return true;
    const double a = -kim;
    auto g = [&](double r) { return std::exp(a * r) / r; };  // 4 pi |G|, up to the common factor
    double hi = std::max(g(rmin), g(rmax)), lo = std::min(g(rmin), g(rmax));
    if (a > 0.0 && 1.0 / a > rmin && 1.0 / a < rmax) lo = std::min(lo, g(1.0 / a));
    const double kabs = std::hypot(kre, kim);
    hi = std::max(hi, kabs);
    lo = std::min(lo, kabs);
    if (kind == 1) {
        const double e1 = std::exp(a * rmin), e2 = std::exp(a * rmax);
        hi = std::max({hi, e1, e2, 1.0});
        lo = std::min({lo, e1, e2, 1.0});
    }
    return !(hi <= lo * (thr / (2.0 * std::sqrt(2.0))));
}

// Items of a job: medium of each, k, the queue order (largest matrices
// first), the amplitude offsets (kind 2), the live count.  Caller holds g_mu.
static int set_items_locked(msgpu_job* J, int nitem, const int* item_med, const double* ks) {
    if (nitem < 1 || nitem > J->cap || !ks) return set_err(MSGPU_E_ARG, "job: bad item count");
    std::vector<int> med_of(nitem);
    double flops = 0.0;
    long long amp_total = 0;
    for (int i = 0; i < nitem; i++) {
        const int mi = item_med ? item_med[i] : 0;
        if (mi < 0 || mi >= J->nmed) return set_err(MSGPU_E_ARG, "job: bad item medium");
        med_of[i] = mi;
        // dlogf jobs always slice six ways (near a root M is ill-conditioned and tr(M^-1 dM/dk)
        // magnifies the factorisation's error by its condition number)
        if (J->precision == MSGPU_MIXED && !J->wide)
            J->wide = J->kind == 1 ||
                      item_may_be_wide(J->med_rmin[mi], J->med_rmax[mi], J->kind, ks[2 * i], ks[2 * i + 1]);
        const double n = J->med_n[mi], n3 = n * n * n, n2 = n * n;
        flops += (J->kind == 0) ? 8.0 / 3.0 * n3
                 : (J->kind == 1 || J->kind == 3) ? (8.0 / 3.0 + 8.0) * n3
                 : (J->kind == 2) ? 8.0 / 3.0 * n3 + 8.0 * n2
                                  : 8.0 / 3.0 * n3 + 50 * 8.0 * n2;  // kind 4: at most 50 solves
        amp_total += J->med_n[mi];
    }
    if ((J->kind == 2 || J->kind == 4) && J->d_amps && amp_total > J->amp_cap)
        return set_err(MSGPU_E_SIZE, "job: amplitudes exceed capacity");
    std::vector<int> order(nitem);
    for (int i = 0; i < nitem; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return J->med_n[med_of[a]] > J->med_n[med_of[b]]; });
    CK(cudaMemcpy(J->d_ks, ks, sizeof(double) * 2 * nitem, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J->d_item_med, med_of.data(), sizeof(int) * nitem, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(J->d_order, order.data(), sizeof(int) * nitem, cudaMemcpyHostToDevice));
    if ((J->kind == 2 || J->kind == 4) && J->d_amp_off) {
        std::vector<long long> off(nitem);
        long long acc = 0;
        for (int i = 0; i < nitem; i++) { off[i] = acc; acc += J->med_n[med_of[i]]; }
        CK(cudaMemcpy(J->d_amp_off, off.data(), sizeof(long long) * nitem, cudaMemcpyHostToDevice));
    }
    const unsigned live = (unsigned)nitem;
    CK(cudaMemcpy(J->d_counter + 1, &live, sizeof(unsigned), cudaMemcpyHostToDevice));
    J->nitem = nitem;
    J->flops = flops;
    J->amp_total = amp_total;
    return 0;
}

msgpu_job* msgpu_job_create(int kind, int nmed, const msgpu_medium* media, int nitem, const int* item_med,
                            const double* ks, int precision) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (init_locked(-1)) return nullptr;
    if (kind < 0 || kind > 4 || nmed < 1 || !media || nitem < 1 || !ks) {
        set_err(MSGPU_E_ARG, "job: bad argument");
        return nullptr;
    }
    if (precision != MSGPU_FP64 && precision != MSGPU_MIXED) {
        set_err(MSGPU_E_ARG, "job: unknown precision");
        return nullptr;
    }
    auto* J = new msgpu_job();
    J->kind = kind;
    J->precision = kind >= 3 ? MSGPU_FP64 : precision;  // traceinv, inverse iteration: FP64 engine
    J->cap = nitem;
    J->nmed = nmed;
    J->med_n.resize(nmed);
    std::vector<MedDev> hm(nmed);
    size_t npos = 0;
    for (int i = 0; i < nmed; i++) {
        const msgpu_medium& m = media[i];
        if (m.n < 1 || m.d < 1 || m.d > 20 || !m.pos || m.n > 50000) {
            set_err(MSGPU_E_ARG, "job: bad medium");
            delete J;
            return nullptr;
        }
        J->nmax = std::max(J->nmax, m.n);
        J->med_n[i] = m.n;
        if (m.d != 3) J->d3only = false;
        npos += (size_t)m.n * m.d;
    }
    // the engine that serves the job (the tuning table may hand a mixed request to the FP64 engine)
    const TuneEntry te = kind < 3 ? g_tune[kind][precision][size_bucket(J->nmax)] : TuneEntry{};
    if (te.engine) J->precision = te.engine - 1;
    // pair-distance range of every d = 3 "maximum" medium (mixed jobs: the entry span of M(k))
    J->med_rmin.assign(nmed, -1.0);
    J->med_rmax.assign(nmed, -1.0);
    if (J->precision == MSGPU_MIXED && kind <= 2)
        for (int i = 0; i < nmed; i++) {
            const msgpu_medium& m = media[i];
            if (m.d != 3 || m.model.type != MSGPU_MAXIMUM || m.n < 2) continue;
            double lo = INFINITY, hi = 0.0;
            for (int a = 0; a < m.n; a++)
                for (int b = a + 1; b < m.n; b++) {
                    const double dx = m.pos[3 * a] - m.pos[3 * b], dy = m.pos[3 * a + 1] - m.pos[3 * b + 1],
                                 dz = m.pos[3 * a + 2] - m.pos[3 * b + 2];
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    lo = std::min(lo, r2);
                    hi = std::max(hi, r2);
                }
            J->med_rmin[i] = std::sqrt(lo);
            J->med_rmax[i] = std::sqrt(hi);
        }
    auto fail = [&](const char* what) -> msgpu_job* {
        set_err(MSGPU_E_CUDA, std::string("job: ") + what);
        msgpu_job_destroy(J);
        return nullptr;
    };
    if (cudaMalloc(&J->d_media, sizeof(MedDev) * nmed) != cudaSuccess) return fail("alloc media");
    if (cudaMalloc(&J->d_pos, sizeof(double) * npos) != cudaSuccess) return fail("alloc pos");
    if (cudaMalloc(&J->d_ks, sizeof(double) * 2 * nitem) != cudaSuccess) return fail("alloc ks");
    if (cudaMalloc(&J->d_item_med, sizeof(int) * nitem) != cudaSuccess) return fail("alloc items");
    if (cudaMalloc(&J->d_order, sizeof(int) * nitem) != cudaSuccess) return fail("alloc order");
    if (cudaMalloc(&J->d_out, sizeof(double) * 2 * nitem) != cudaSuccess) return fail("alloc out");
    if (cudaMalloc(&J->d_status, sizeof(int) * nitem) != cudaSuccess) return fail("alloc status");
    if (cudaMalloc(&J->d_counter, 256) != cudaSuccess) return fail("alloc counter");
    if (cudaMemset(J->d_counter, 0, 256) != cudaSuccess) return fail("clear counter");
    if (kind == 2 || kind == 4) {
        // capacity for the amplitudes (eigenvectors) of nitem items of the largest medium
        J->amp_cap = (long long)nitem * J->nmax;
        if (cudaMalloc(&J->d_amps, sizeof(double) * 2 * (size_t)J->amp_cap) != cudaSuccess) return fail("alloc amps");
        if (cudaMalloc(&J->d_amp_off, sizeof(long long) * nitem) != cudaSuccess) return fail("alloc amp_off");
    }
    size_t off = 0;
    for (int i = 0; i < nmed; i++) {
        const msgpu_medium& m = media[i];
        size_t cnt = (size_t)m.n * m.d;
        if (cudaMemcpy(J->d_pos + off, m.pos, sizeof(double) * cnt, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail("copy pos");
        hm[i] = MedDev{m.d, m.n, J->d_pos + off, m.model};
        off += cnt;
    }
    if (cudaMemcpy(J->d_media, hm.data(), sizeof(MedDev) * nmed, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail("copy media");
    if (set_items_locked(J, nitem, item_med, ks)) {
        msgpu_job_destroy(J);
        return nullptr;
    }
    // per-CTA slots
    J->slot = (size_t)J->nmax * J->nmax;
    const size_t per_cta = slot_elems(kind, J->slot, J->nmax) * sizeof(zc);
    const int ctas = te.ctas ? std::min(te.ctas, g_ctas_fp64) : g_ctas_fp64;
    int grid = std::min(nitem, g_sms * ctas);
    size_t budget = ws_budget();
    while (grid > 1 && (size_t)grid * per_cta > budget) grid--;
    J->grid = grid;
    J->ws_bytes = (size_t)grid * per_cta;
    if (cudaMalloc(&J->d_piv, sizeof(int) * (size_t)grid * J->nmax) != cudaSuccess) return fail("alloc piv");
    void* ws = nullptr;
    if (ensure_ws(J->ws_bytes, &ws)) {
        msgpu_job_destroy(J);
        return nullptr;
    }
    return J;
}

int msgpu_job_set_points(msgpu_job* J, int nitem, const int* item_med, const double* ks) {
    if (!J) return set_err(MSGPU_E_ARG, "null job");
    std::lock_guard<std::mutex> lk(g_mu);
    return set_items_locked(J, nitem, item_med, ks);
}

int msgpu_job_use_graph(msgpu_job* J, int on) {
    if (!J) return set_err(MSGPU_E_ARG, "null job");
    std::lock_guard<std::mutex> lk(g_mu);
    J->use_graph = on != 0;
    return 0;
}

// the work of one run on stream st: reset the queue, launch the engine
static int launch_locked(msgpu_job* J, void* ws, cudaStream_t st) {
    CK(cudaMemsetAsync(J->d_counter, 0, sizeof(unsigned), st));
    EngineParams P;
    P.media = J->d_media;
    P.ks = J->d_ks;
    P.item_med = J->d_item_med;
    P.order = J->d_order;
    P.nitem = J->cap;
    P.ws = reinterpret_cast<zc*>(ws);
    P.slot = J->slot;
    P.piv = J->d_piv;
    P.piv_stride = J->nmax;
    P.out = J->d_out;
    P.status = J->d_status;
    P.counter = J->d_counter;
    P.kind = J->kind;
    P.wide_ok = J->wide ? 1 : 0;
    P.warm = J->warm ? 1 : 0;
    P.amps = J->d_amps;
    P.amp_off = J->d_amp_off;
    if (J->precision == MSGPU_MIXED) {
        int e = mixed_run(P, J->grid, J->nmax, J->d3only, st);
        if (e) return set_err(e, "mixed engine launch failed");
        return 0;
    }
    k_engine_fp64<<<J->grid, NT, smem_bytes(), st>>>(P);
    CK(cudaGetLastError());
    return 0;
}

int msgpu_job_run(msgpu_job* J, void* stream) {
    if (!J) return set_err(MSGPU_E_ARG, "null job");
    std::lock_guard<std::mutex> lk(g_mu);
    cudaStream_t st = (cudaStream_t)stream;
    void* ws = nullptr;
    if (int e = ensure_ws(J->ws_bytes, &ws)) return e;
    if (!J->use_graph) {
        if (int e = launch_locked(J, ws, st)) return e;
        g_launches++;
        return 0;
    }
    if (J->precision == MSGPU_MIXED && mixed_prepare(J->grid, J->nmax)) return set_err(MSGPU_E_CUDA, "mixed scratch");
    // the graph holds the workspace and scratch addresses, the launch's shared-memory size
    // (wide) and the start-vector mode (warm)
    const unsigned long long gen =
        ((g_ws_gen * 0x9E3779B97F4A7C15ULL + mixed_generation()) * 2 + (J->wide ? 1 : 0)) * 2 + (J->warm ? 1 : 0);
    if (!J->gexec || J->gen != gen) {
        // (re)capture: the graph holds the workspace and scratch addresses
        if (J->gexec) cudaGraphExecDestroy(J->gexec);
        J->gexec = nullptr;
        if (!J->cap_stream) CK(cudaStreamCreateWithFlags(&J->cap_stream, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(J->cap_stream, cudaStreamCaptureModeRelaxed));
        const int e = launch_locked(J, ws, J->cap_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(J->cap_stream, &g);
        if (e) {
            if (g) cudaGraphDestroy(g);
            return e;
        }
        CK(ce);
        const cudaError_t ie = cudaGraphInstantiate(&J->gexec, g, 0);
        cudaGraphDestroy(g);
        CK(ie);
        J->gen = gen;
    }
    CK(cudaGraphLaunch(J->gexec, st));
    g_launches++;
    return 0;
}

int msgpu_job_launches(const msgpu_job* J) { return J ? 1 : 0; }

int msgpu_engine_stats(double* out, int n) { return mixed_stats(out, n); }
double msgpu_job_flops(const msgpu_job* J) { return J ? J->flops : 0.0; }

int msgpu_job_results(msgpu_job* J, double* out, int* status) {
    if (!J) return set_err(MSGPU_E_ARG, "null job");
    CK(cudaDeviceSynchronize());
    if (out) CK(cudaMemcpy(out, J->d_out, sizeof(double) * 2 * J->nitem, cudaMemcpyDeviceToHost));
    if (status) CK(cudaMemcpy(status, J->d_status, sizeof(int) * J->nitem, cudaMemcpyDeviceToHost));
    return 0;
}

int msgpu_job_amplitudes(msgpu_job* J, double* amps) {
    if (!J || (J->kind != 2 && J->kind != 4) || !amps)
        return set_err(MSGPU_E_ARG, "job_amplitudes: not an amplitude or eigenvector job");
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(amps, J->d_amps, sizeof(double) * 2 * (size_t)J->amp_total, cudaMemcpyDeviceToHost));
    return 0;
}

int msgpu_job_set_vectors(msgpu_job* J, const double* vecs) {
    if (!J || J->kind != 4 || !vecs || !J->d_amps)
        return set_err(MSGPU_E_ARG, "job_set_vectors: not an eigenvector job");
    std::lock_guard<std::mutex> lk(g_mu);
    CK(cudaMemcpy(J->d_amps, vecs, sizeof(double) * 2 * (size_t)J->amp_total, cudaMemcpyHostToDevice));
    J->warm = true;
    return 0;
}

void msgpu_job_destroy(msgpu_job* J) {
    if (!J) return;
    if (J->gexec) cudaGraphExecDestroy(J->gexec);
    if (J->cap_stream) cudaStreamDestroy(J->cap_stream);
    cudaFree(J->d_media);
    cudaFree(J->d_pos);
    cudaFree(J->d_ks);
    cudaFree(J->d_item_med);
    cudaFree(J->d_order);
    cudaFree(J->d_out);
    cudaFree(J->d_status);
    cudaFree(J->d_counter);
    cudaFree(J->d_piv);
    cudaFree(J->d_amps);
    cudaFree(J->d_amp_off);
    delete J;
}

int msgpu_tune_set(int kind, int precision, int n, int engine, int ctas_per_sm) {
    if (kind < 0 || kind > 2 || (precision != MSGPU_FP64 && precision != MSGPU_MIXED) || n < 1 ||
        (engine != -1 && engine != MSGPU_FP64 && engine != MSGPU_MIXED) || ctas_per_sm < 0 || ctas_per_sm > 8)
        return set_err(MSGPU_E_ARG, "tune_set: bad argument");
    if (precision == MSGPU_FP64 && engine == MSGPU_MIXED)
        return set_err(MSGPU_E_ARG, "tune_set: an FP64 request cannot run on the mixed engine");
    std::lock_guard<std::mutex> lk(g_mu);
    TuneEntry& e = g_tune[kind][precision][size_bucket(n)];
    e.engine = engine < 0 ? 0 : engine + 1;
    e.ctas = ctas_per_sm;
    return 0;
}

int msgpu_tune_get(int kind, int precision, int n, int* engine, int* ctas_per_sm) {
    if (kind < 0 || kind > 2 || (precision != MSGPU_FP64 && precision != MSGPU_MIXED) || n < 1 || !engine ||
        !ctas_per_sm)
        return set_err(MSGPU_E_ARG, "tune_get: bad argument");
    std::lock_guard<std::mutex> lk(g_mu);
    const TuneEntry& e = g_tune[kind][precision][size_bucket(n)];
    *engine = e.engine - 1;
    *ctas_per_sm = e.ctas;
    return 0;
}

int msgpu_autotune(int kind, int precision, int d, int n, int nitem, double* seconds) {
    if (kind < 0 || kind > 2 || (precision != MSGPU_FP64 && precision != MSGPU_MIXED) || d < 2 || d > 3 ||
        n < 2 || nitem < 1 || !seconds)
        return set_err(MSGPU_E_ARG, "autotune: bad argument");
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (int e = init_locked(-1)) return e;
    }
    // probe: n scatterers of the reference's ball (seed 1), nitem k on the
    // real axis ... -0.05i (cross sections need real k)
    std::vector<double> pos((size_t)n * d), ks(2 * (size_t)nitem);
    if (int e = msgpu_fill_medium(d, n, MSGPU_BALL, 1.0, 1, pos.data())) return e;
    for (int i = 0; i < nitem; ++i) {
        ks[2 * i] = 0.5 + 2.5 * i / std::max(1, nitem - 1);
        ks[2 * i + 1] = kind == 2 ? 0.0 : -0.05;
    }
    const msgpu_medium med{d, n, pos.data(), {MSGPU_MAXIMUM, 0, {0.0, 0.0}}};
    const int engines[2] = {MSGPU_FP64, MSGPU_MIXED};
    double best = 0.0;
    int best_e = precision, best_c = 0;
    for (int ei = 0; ei < (precision == MSGPU_MIXED ? 2 : 1); ++ei)
        for (int c = 1; c <= 2; ++c) {
            const int eng = precision == MSGPU_MIXED ? engines[ei] : MSGPU_FP64;
            double& t = seconds[ei * 2 + (c - 1)];
            t = -1.0;
            if (c > g_ctas_fp64) continue;
            if (int e = msgpu_tune_set(kind, precision, n, eng, c)) return e;
            msgpu_job* J = msgpu_job_create(kind, 1, &med, nitem, nullptr, ks.data(), precision);
            if (!J) return MSGPU_E_CUDA;
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            int err = msgpu_job_run(J, nullptr);  // warm-up (allocations, first launch)
            if (!err) err = cudaDeviceSynchronize() == cudaSuccess ? 0 : MSGPU_E_CUDA;
            float ms = 0.0f;
            if (!err) {
                cudaEventRecord(e0, nullptr);
                err = msgpu_job_run(J, nullptr);
                cudaEventRecord(e1, nullptr);
                if (!err && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            msgpu_job_destroy(J);
            if (err) return err;
            t = 1e-3 * ms;
            if (best == 0.0 || t < best) {
                best = t;
                best_e = eng;
                best_c = c;
            }
        }
    return msgpu_tune_set(kind, precision, n, best_e, best_c);
}

static int run_batch(int kind, int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                     double* out, int* status, int precision) {
    msgpu_job* J = msgpu_job_create(kind, nmed, media, nitem, item_med, ks, precision);
    if (!J) return g_err.empty() ? MSGPU_E_ARG : (g_err.find("CUDA") != std::string::npos ? MSGPU_E_CUDA : MSGPU_E_ARG);
    int e = msgpu_job_run(J, nullptr);
    if (!e) e = msgpu_job_results(J, out, status);
    msgpu_job_destroy(J);
    return e;
}

int msgpu_tracelog_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                         double* out, int* status, int precision) {
    return run_batch(0, nmed, media, nitem, item_med, ks, out, status, precision);
}

int msgpu_dk_log_det_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                           double* out, int* status, int precision) {
    return run_batch(1, nmed, media, nitem, item_med, ks, out, status, precision);
}

int msgpu_traceinv_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                         double* out, int* status, int precision) {
    return run_batch(3, nmed, media, nitem, item_med, ks, out, status, precision);
}

int msgpu_inverse_iteration_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med,
                                  const double* ks, double* lambda, double* vecs, int* status, int precision) {
    msgpu_job* J = msgpu_job_create(4, nmed, media, nitem, item_med, ks, precision);
    if (!J) return MSGPU_E_ARG;
    int e = msgpu_job_run(J, nullptr);
    if (!e) e = msgpu_job_results(J, lambda, status);
    if (!e && vecs) e = msgpu_job_amplitudes(J, vecs);
    msgpu_job_destroy(J);
    return e;
}

int msgpu_amplitude_batch(int nmed, const msgpu_medium* media, int nitem, const int* item_med, const double* ks,
                          double* out, double* amps, int* status, int precision) {
    msgpu_job* J = msgpu_job_create(2, nmed, media, nitem, item_med, ks, precision);
    if (!J) return MSGPU_E_ARG;
    int e = msgpu_job_run(J, nullptr);
    if (!e) e = msgpu_job_results(J, out, status);
    if (!e && amps) e = msgpu_job_amplitudes(J, amps);
    msgpu_job_destroy(J);
    return e;
}

}  // extern "C"
