#include "profiler.cuh"

namespace forge {

static thread_local Profiler* g_prof = nullptr;
Profiler* current_profiler() { return g_prof; }
void set_current_profiler(Profiler* p) { g_prof = p; }

cudaEvent_t Profiler::get() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Profiler::begin(int stage) {
    open_stage = stage;
    open_ev = get();
    cudaEventRecord(open_ev, stream);
}

void Profiler::end(int stage, double b, double f) {
    if (open_stage != stage || !open_ev) return;
    cudaEvent_t e = get();
    cudaEventRecord(e, stream);
    pending.push_back({stage, open_ev, e, b, f});
    open_ev = nullptr;
    open_stage = -1;
    if (pending.size() > 16384) collect();
}

int Profiler::collect() {
    if (pending.empty()) return 0;
    cudaStreamSynchronize(stream);
    for (auto& p : pending) {
        float t = 0.f;
        cudaEventElapsedTime(&t, p.a, p.b);
        ms[p.stage] += t;
        bytes[p.stage] += p.bytes;
        flops[p.stage] += p.flops;
        launches[p.stage] += 1;
        pool.push_back(p.a);
        pool.push_back(p.b);
    }
    pending.clear();
    return 0;
}

void Profiler::reset() {
    collect();
    for (int s = 0; s < ST_COUNT; ++s) {
        ms[s] = bytes[s] = flops[s] = 0.0;
        launches[s] = 0;
    }
}

void Profiler::release() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto& p : pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    pending.clear();
    for (auto e : pool) cudaEventDestroy(e);
    pool.clear();
    if (open_ev) cudaEventDestroy(open_ev);
    open_ev = nullptr;
}

}  // namespace forge
