// mixed.cu -- host side of the mixed-precision engine: its per-CTA scratch,
// the launch of the variant a job needs, the phase statistics, and the
// tensor-core layout probe.  The device side (slicing, tcgen05 trailing
// update, double-float panel and TRSM, assembly, solves) is mixed_engine.cuh;
// the kernel variants are instantiated in the mixed_k*.cu units.
#include "mixed_engine.cuh"

namespace msg {

// ---------------------------------------------------------------- host side
namespace {
std::mutex g_mx;
uint8_t* g_img = nullptr;
size_t g_img_bytes = 0;
int* g_err = nullptr;
unsigned long long* g_stats = nullptr;
int g_first_wait = WAIT_LIMIT;
}  // namespace

// the operand buffers need 16-byte alignment (no-swizzle layout); 128 is kept
static size_t mixed_smem() { return MIX_SMEM_WIDE; }

using Variant = int (*)(const EngineParams&, const MixScratch&, int, size_t, cudaStream_t, bool);
const Variant kVariants[6] = {mixed_variant_0_d3, mixed_variant_1_d3, mixed_variant_2_d3,
                              mixed_variant_0_any, mixed_variant_1_any, mixed_variant_2_any};

unsigned long long g_mix_gen = 1;

// scratch layout for `grid` CTAs and matrices up to nmax; allocates when it grows
static int prepare_locked(int grid, int nmax, MixScratch& X) {
    static bool attr = false;
    if (!attr) {
        const int sm = (int)mixed_smem();
        for (auto f : kVariants)
            if (f(EngineParams{}, MixScratch{}, 0, (size_t)sm, nullptr, true)) return MSGPU_E_CUDA;
        attr = true;
    }
    // images sized for the larger of the two slice configurations
    const int nbA = (nmax + MT_M - 1) / MT_M, ncB = (nmax + 31) / 32 * 32;
    X.a_stride = (size_t)nbA * A_IMG_BAND;
    X.b_stride = (size_t)ncB * B_IMG_COL;
    X.e_stride = (size_t)nbA * MT_M + 32;
    const size_t need = (size_t)grid * (X.a_stride + X.b_stride) + 2 * sizeof(float) * grid * X.e_stride + 256;
    if (need > g_img_bytes) {
        if (g_img) cudaFree(g_img);
        g_img = nullptr;
        g_img_bytes = 0;
        ++g_mix_gen;
        if (cudaMalloc(&g_img, need) != cudaSuccess) return MSGPU_E_CUDA;
        g_img_bytes = need;
    }
    if (!g_err) {
        ++g_mix_gen;
        if (cudaMalloc(&g_err, sizeof(int)) != cudaSuccess) return MSGPU_E_CUDA;
    }
    if (getenv("MSGPU_STATS") && !g_stats) {
        ++g_mix_gen;
        if (cudaMalloc(&g_stats, sizeof(unsigned long long) * PH_N) != cudaSuccess) return MSGPU_E_CUDA;
    }
    X.imgA = g_img;
    X.imgB = g_img + (size_t)grid * X.a_stride;
    X.ea = reinterpret_cast<float*>(X.imgB + (size_t)grid * X.b_stride);
    X.eb = X.ea + (size_t)grid * X.e_stride;
    X.err = g_err;
    X.stats = getenv("MSGPU_STATS") ? g_stats : nullptr;
    X.first_wait = g_first_wait;
    return 0;
}

int mixed_prepare(int grid, int nmax) {
    std::lock_guard<std::mutex> lk(g_mx);
    MixScratch X;
    return prepare_locked(grid, nmax, X);
}

unsigned long long mixed_generation() {
    std::lock_guard<std::mutex> lk(g_mx);
    return g_mix_gen;
}

int mixed_run(const EngineParams& P, int grid, int nmax, bool d3only, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_mx);
    MixScratch X;
    if (int e = prepare_locked(grid, nmax, X)) return e;
    if (X.stats) cudaMemsetAsync(X.stats, 0, sizeof(unsigned long long) * PH_N, st);
    if (cudaMemsetAsync(P.counter, 0, sizeof(unsigned), st) != cudaSuccess) return MSGPU_E_CUDA;
    // variants: kinds 0..2 for media all of d = 3, then for any dimension
    const int v = (d3only ? 0 : 3) + (P.kind < 0 ? 0 : P.kind > 2 ? 2 : P.kind);
    return kVariants[v](P, X, grid, P.wide_ok ? MIX_SMEM_WIDE : MIX_SMEM_NARROW, st, false);
}

int mixed_stats(double* out, int n) {
    if (!g_stats) return 0;
    unsigned long long h[PH_N];
    if (cudaMemcpy(h, g_stats, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return MSGPU_E_CUDA;
    for (int i = 0; i < n && i < PH_N; ++i) out[i] = (double)h[i];
    return PH_N;
}

// ---------------------------------------------------------------- layout self-check
__global__ void __launch_bounds__(128, 1) k_probe_umma(const float* A, const float* B, float* D, int mode,
                                                       int* err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t* As = sm;
    uint8_t* Bs = sm + 16384;
    for (int i = tid; i < 65536 / 16; i += 128) reinterpret_cast<int4*>(sm)[i] = make_int4(0, 0, 0, 0);
    __syncthreads();
    for (int e = tid; e < 128 * 32; e += 128) {
        int r = e / 32, k = e % 32;
        *reinterpret_cast<__nv_bfloat16*>(As + cm_offset(r, k, 128)) = __float2bfloat16_rn(A[e]);
    }
    for (int e = tid; e < 64 * 32; e += 128) {
        int r = e / 32, k = e % 32;
        *reinterpret_cast<__nv_bfloat16*>(Bs + cm_offset(r, k, 64)) = __float2bfloat16_rn(B[e]);
    }
    if (warp == 0) {
        tmem_alloc(&tbase, 64);
        tmem_relinquish();
    }
    if (tid == 0) mbar_init(&bar, 1);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tbase;
    if (tid == 0) {
        uint32_t a0 = smem_u32(As), b0 = smem_u32(Bs);
        uint32_t lboA = 2048, sboA = 128, lboB = 1024, sboB = 128;
        if (mode & 1) {
            lboA = 128; sboA = 2048; lboB = 128; sboB = 1024;
        }
        const uint32_t id = idesc_bf16(128, 64, false, (mode & 2) != 0);
        for (int ks = 0; ks < 2; ++ks)
            umma_bf16(tmem, sdesc(a0 + ks * 4096, lboA, sboA), sdesc(b0 + ks * 2048, lboB, sboB), id, ks > 0);
        umma_commit(&bar);
    }
    const bool ok = mbar_wait(&bar, 0);
    if (!ok && lane == 0) atomicExch(err, 1);
    tc_fence_after();
    float v[32];
    for (int half = 0; half < 2; ++half) {
        tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + half * 32, v);
        tmem_wait_ld();
        for (int j = 0; j < 32; ++j) D[(32 * warp + lane) * 64 + half * 32 + j] = v[j];
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 64);
}

}  // namespace msg

// Poll limit of the first operand wait of every mixed trailing update in later
// runs (polls < 0: the normal limit).  A test sets 0 to make that wait run out
// and checks that the items report MSGPU_S_TIMEOUT and the context stays usable.
extern "C" int msgpu_debug_first_wait_limit(int polls) {
    std::lock_guard<std::mutex> lk(msg::g_mx);
    msg::g_first_wait = polls < 0 ? msg::WAIT_LIMIT : polls;
    ++msg::g_mix_gen;  // captured runs hold the old limit: recapture them
    return 0;
}

extern "C" int msgpu_probe_umma(int mode, const float* A, const float* B, float* D) {
    using namespace msg;
    if (msgpu_init(-1)) return MSGPU_E_NODEV;
    float *dA = nullptr, *dB = nullptr, *dD = nullptr;
    int* derr = nullptr;
    int herr = 0;
    auto done = [&](int rc) {
        cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(derr);
        return rc;
    };
    if (cudaMalloc(&dA, 128 * 32 * 4) || cudaMalloc(&dB, 64 * 32 * 4) || cudaMalloc(&dD, 128 * 64 * 4) ||
        cudaMalloc(&derr, 4))
        return done(MSGPU_E_CUDA);
    if (cudaMemcpy(dA, A, 128 * 32 * 4, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dB, B, 64 * 32 * 4, cudaMemcpyHostToDevice) || cudaMemset(dD, 0, 128 * 64 * 4) ||
        cudaMemset(derr, 0, 4) || cudaFuncSetAttribute(k_probe_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, 65536))
        return done(MSGPU_E_CUDA);
    k_probe_umma<<<1, 128, 65536>>>(dA, dB, dD, mode, derr);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(D, dD, 128 * 64 * 4, cudaMemcpyDeviceToHost) || cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost))
        return done(MSGPU_E_CUDA);
    return done(herr ? MSGPU_E_CUDA : 0);
}
