// engine_internal.h -- structures shared by the engine translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "msgpu.h"
#include "cplx.cuh"
#include "error_text.h"

namespace msg {

struct MedDev {
    int d, n;
    const double* pos;
    msgpu_model model;
};

struct EngineParams {
    const MedDev* media;
    const double* ks;     // 2 * nitem
    const int* item_med;  // nitem
    const int* order;     // queue position -> item index
    int nitem;
    zc* ws;               // per-CTA slots
    size_t slot;          // complex elements per matrix slot
    int* piv;             // per-CTA pivots
    int piv_stride;
    double* out;          // 2 * nitem
    int* status;          // nitem
    unsigned* counter;    // [0] work queue; [1] live items (queue positions >= it are past the end)
    int kind;             // 0 ln det / n, 1 dlogf, 2 amplitudes a = M^-1 phi, 3 traceinv, 4 inverse iteration
    double* amps;         // kinds 2, 4: a (or the eigenvector) per item (2 * n_i doubles each) or nullptr
    const long long* amp_off;  // kind 2: offset (in complex elements) of item i in amps
    int wide_ok;          // mixed engine: the launch has the shared memory for six-way slicing
    int warm;             // kind 4: start each inverse iteration from the item's vector in amps
};


// adds to the library's count of kernel launches (msgpu_launch_count)
void count_launches(int n);

// Mixed-precision engine (mixed.cu).  Returns 0 when it ran the job, a
// negative MSGPU_E* code on error.
// d3only: every medium of the job has d = 3 (selects the d = 3 kernel instantiation);
// P.wide_ok: launch with the shared memory for six-way slicing.
int mixed_run(const EngineParams& P, int grid, int nmax, bool d3only, cudaStream_t st);
// Allocates the mixed engine's scratch for `grid` CTAs and matrices up to nmax
// (mixed_run does so itself; called before a stream capture, which must not allocate).
int mixed_prepare(int grid, int nmax);
// Changes whenever the mixed engine's scratch is reallocated (captured graphs hold its address).
unsigned long long mixed_generation();
// per-phase SM cycles of the last mixed run made with MSGPU_STATS set:
// assemble, panel, trsm, slice, tiles, solve, items
int mixed_stats(double* out, int n);

}  // namespace msg
