// noalloc.cu -- ln det M(k)/n for callers that cannot allocate device memory.
//
// Some hosts of this library must not call cudaMalloc at all: code running
// under a CUDA graph being captured, inside a memory pool that another
// runtime owns, or in a process whose device memory is carved up in advance
// (an embedding application that reserves the whole GPU for its own
// allocator).  msgpu_tracelog_batch_noalloc serves them: the caller passes
// device pointers for inputs and outputs, and every byte of scratch the FP64
// engine needs (its per-CTA matrix slots, pivots, the work-queue counter and
// the item tables) comes from one file-scope __device__ array of fixed size,
// NOALLOC_BYTES, which every GPU that loads the library holds until the
// process exits.  Nothing here calls cudaMalloc, cudaFree or an allocating
// library routine.
//
// Sharing rules: every call uses the same array and it keeps the previous
// call's contents; the set-up kernel clears what must start at zero (the
// work counter) on every call.  Calls whose kernels overlap on the GPU race
// on the array: issue them on one stream, or order them.  The first call on
// a device looks up the array's device address (cudaGetSymbolAddress) and
// sets the engine kernel's shared-memory attribute; make that first call
// before any stream capture begins.
#include <cuda_runtime.h>
#include <mutex>
#include "engine_internal.h"
#include "lu64.cuh"

namespace msg {

// the FP64 engine kernel (engine.cu), launched here on the static scratch
__global__ void __launch_bounds__(NT, 2) k_engine_fp64(EngineParams P);

constexpr size_t NOALLOC_BYTES = (size_t)128 << 20;  // 128 MiB per device
constexpr int NOALLOC_MAX_ITEMS = 1 << 16;
constexpr int NOALLOC_MAX_N = 2048;
constexpr size_t NOALLOC_HEADER = 512 + 2 * sizeof(int) * (size_t)NOALLOC_MAX_ITEMS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

__global__ void k_noalloc_setup(MedDev* md, MedDev v, unsigned* counter, int* item_med, int* order, int nitem) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *md = v;
        counter[0] = 0u;
        counter[1] = (unsigned)nitem;  // live items of the work queue
    }
    for (; i < nitem; i += gridDim.x * blockDim.x) {
        item_med[i] = 0;
        order[i] = i;
    }
}

namespace {
std::mutex g_na_mu;
void* g_na_addr[64] = {nullptr};
int g_na_sms[64] = {0};
}  // namespace

}  // namespace msg

extern "C" int msgpu_tracelog_batch_noalloc(int d, int n, const double* d_pos, msgpu_model model, int nk,
                                            const double* d_ks, double* d_out, int* d_status, void* stream) {
    using namespace msg;
    if (d < 1 || d > 20 || n < 1 || nk < 1 || !d_pos || !d_ks || !d_out || !d_status)
        return record_error(MSGPU_E_ARG, "noalloc: bad argument (d in 1..20, n >= 1, nk >= 1, non-null pointers)");
    if (n > NOALLOC_MAX_N || nk > NOALLOC_MAX_ITEMS)
        return record_error(MSGPU_E_SIZE, "noalloc: n > 2048 or nk > 65536 exceeds the fixed scratch array");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return record_error(MSGPU_E_NODEV, "noalloc: cudaGetDevice failed or device index beyond 63");
    void* base = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
                return record_error(MSGPU_E_CUDA, "noalloc: cudaGetSymbolAddress of the scratch array failed");
            if (cudaFuncSetAttribute(k_engine_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(LuSmem)) != cudaSuccess)
                return record_error(MSGPU_E_CUDA, "noalloc: cudaFuncSetAttribute(k_engine_fp64) failed");
            int nsm = 0;
            if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
                return record_error(MSGPU_E_CUDA, "noalloc: cudaDeviceGetAttribute(SM count) failed");
            g_na_sms[dev] = nsm;
            g_na_addr[dev] = p;
        }
        base = g_na_addr[dev];
        sms = g_na_sms[dev];
    }
    unsigned char* b = static_cast<unsigned char*>(base);
    MedDev* md = reinterpret_cast<MedDev*>(b);
    unsigned* counter = reinterpret_cast<unsigned*>(b + 256);
    int* item_med = reinterpret_cast<int*>(b + 512);
    int* order = item_med + NOALLOC_MAX_ITEMS;
    const size_t slot = (size_t)n * n;                       // complex elements per CTA slot
    const size_t per_cta = slot * sizeof(zc) + (((size_t)n * sizeof(int) + 255) / 256) * 256;
    size_t grid = (NOALLOC_BYTES - NOALLOC_HEADER - 256) / per_cta;
    if (grid > (size_t)(2 * sms)) grid = 2 * sms;
    if (grid > (size_t)nk) grid = nk;
    if (grid < 1) return record_error(MSGPU_E_SIZE, "noalloc: one matrix slot does not fit the scratch array");
    const size_t ws_off = (NOALLOC_HEADER + 255) / 256 * 256;
    zc* ws = reinterpret_cast<zc*>(b + ws_off);
    int* piv = reinterpret_cast<int*>(b + ws_off + grid * slot * sizeof(zc));
    cudaStream_t st = (cudaStream_t)stream;
    MedDev v{d, n, d_pos, model};
    k_noalloc_setup<<<(nk + 255) / 256, 256, 0, st>>>(md, v, counter, item_med, order, nk);
    if (cudaGetLastError() != cudaSuccess) return record_error(MSGPU_E_CUDA, "noalloc: set-up kernel launch failed");
    EngineParams P;
    P.media = md;
    P.ks = d_ks;
    P.item_med = item_med;
    P.order = order;
    P.nitem = nk;
    P.ws = ws;
    P.slot = slot;
    P.piv = piv;
    P.piv_stride = n;
    P.out = d_out;
    P.status = d_status;
    P.counter = counter;
    P.kind = 0;
    P.amps = nullptr;
    P.amp_off = nullptr;
    P.wide_ok = 0;
    P.warm = 0;
    k_engine_fp64<<<(unsigned)grid, NT, sizeof(LuSmem), st>>>(P);
    if (cudaGetLastError() != cudaSuccess) return record_error(MSGPU_E_CUDA, "noalloc: engine kernel launch failed");
    count_launches(2);
    return 0;
}
