// Per-stage CUDA-event timing on the context's stream (off unless enabled).
//
// Each tracked launch is bracketed by two events from a reusable pool; the host sums
// the elapsed times per stage when the profile is read, together with the launch
// count and the algorithmic bytes / flops the call sites declare per launch.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace forge {

enum ProfStage {
    ST_TABLES = 0,
    ST_LR,
    ST_ASSEMBLE,
    ST_TRD_COL,
    ST_HEMV,
    ST_TRD_FINISH,
    ST_HER2K,
    ST_BISECT,
    ST_INVIT,
    ST_BACKTRANSFORM,
    ST_PROJECTOR,
    ST_WINDOW,
    ST_SORT,
    ST_ENERGY,
    ST_LRMATVEC,
    ST_MIX,
    ST_REFINE,
    ST_OA_GEMM,   // sliced (error-free) residual product H X of the eigenpair refinement
    ST_OA,        // the refinement's other steps: slices, overlaps, correction, update
    ST_COUNT
};

struct Profiler {
    bool enabled = false;
    struct Pending {
        int stage;
        cudaEvent_t a, b;
        double bytes, flops;
    };
    std::vector<cudaEvent_t> pool;
    std::vector<Pending> pending;
    double ms[ST_COUNT] = {}, bytes[ST_COUNT] = {}, flops[ST_COUNT] = {};
    int64_t launches[ST_COUNT] = {};
    cudaStream_t stream = nullptr;
    int open_stage = -1;
    cudaEvent_t open_ev = nullptr;

    cudaEvent_t get();
    void begin(int stage);
    void end(int stage, double bytes, double flops);
    int collect();  // synchronises and folds pending pairs into the totals
    void reset();
    void release();
};

// the profiler of the context currently executing a C-ABI call (thread-local)
Profiler* current_profiler();
void set_current_profiler(Profiler* p);

inline void prof_begin(int stage) {
    Profiler* p = current_profiler();
    if (p && p->enabled) p->begin(stage);
}
inline void prof_end(int stage, double bytes, double flops) {
    Profiler* p = current_profiler();
    if (p && p->enabled) p->end(stage, bytes, flops);
}

}  // namespace forge
