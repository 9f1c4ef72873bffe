// Allocation-free variant of the FP64 partial Hermitian eigen-solver (zdiagRed,
// LapackRoutines.f90:381-433, for one matrix).
//
// Some callers cannot allocate device memory at call time: code running inside a memory
// pool or arena that owns every byte of the GPU, and hosts that manage all device buffers
// themselves and hand this library only pointers.  forge_gpu_zheevr_noalloc serves them: the
// caller passes device pointers for its input and outputs and a stream, and the solver's
// workspace lives in the file-scope device array below, sized for matrices up to
// FORGE_NOALLOC_MAX_N (512).  Every GPU that loads this library holds that array
// (FORGE_NOALLOC_SCRATCH_BYTES) until the process exits.
//
// The array is shared by every call on a device and keeps the contents of the last call; the
// solver clears what must start at zero (its CTA counters and the failure flags) at the start of
// each call.  Calls whose work overlaps on the GPU race on the array, so callers must order
// them (one stream, or events).  Host code only uses the array through the device address
// obtained with cudaGetSymbolAddress, once per device with that device current, during the
// first call on that device (std::call_once per device: concurrent first calls from several
// host threads look it up once).  Each call synchronises its stream at the end to read the
// solver's convergence flag, so it blocks the host and cannot be recorded into a CUDA graph.
// The call hides its work from the calling thread's context profiler (a thread-local pointer)
// for its duration, since profiling would create events.
#include <cstring>
#include <mutex>

#include "eig.cuh"

namespace forge {

constexpr int64_t kNoAllocMaxN = FORGE_NOALLOC_MAX_N;
constexpr size_t kNoAllocBytes = FORGE_NOALLOC_SCRATCH_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// device address of g_noalloc_scratch per device, looked up once per device
static void* g_noalloc_ptr[64] = {};
static cudaError_t g_noalloc_err[64] = {};
static std::once_flag g_noalloc_once[64];

}  // namespace forge

using namespace forge;

extern "C" int forge_gpu_zheevr_noalloc(double* A, int64_t n, int64_t iu, double* w, double* Z, void* stream) {
    if (!A || !w || !Z || n < 2 || iu < 1 || iu > n) {
        set_error(FORGE_ERR_ARG, "zheevr_noalloc: bad arguments (need device A, w, Z, n >= 2, 1 <= iu <= n)");
        return FORGE_ERR_ARG;
    }
    if (n > kNoAllocMaxN) {
        set_error(FORGE_ERR_ARG, "zheevr_noalloc: n = %lld exceeds the allocation-free maximum of %lld",
                  (long long)n, (long long)kNoAllocMaxN);
        return FORGE_ERR_ARG;
    }
    const size_t need = eig_workspace_bytes(n, iu, 1);
    if (need > kNoAllocBytes) {
        set_error(FORGE_ERR_ARG, "zheevr_noalloc: workspace of %zu bytes exceeds the %zu-byte static array", need,
                  kNoAllocBytes);
        return FORGE_ERR_ARG;
    }
    int dev = 0;
    FORGE_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error(FORGE_ERR_ARG, "zheevr_noalloc: device ordinal %d out of range", dev);
        return FORGE_ERR_ARG;
    }
    std::call_once(g_noalloc_once[dev], [dev]() {
        void* p = nullptr;
        g_noalloc_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        g_noalloc_ptr[dev] = p;
    });
    if (g_noalloc_err[dev] != cudaSuccess || !g_noalloc_ptr[dev]) {
        set_error(FORGE_ERR_CUDA, "zheevr_noalloc: cudaGetSymbolAddress of the static workspace failed: %s",
                  cudaGetErrorString(g_noalloc_err[dev]));
        return FORGE_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // no context profiler records into this call (it would create events)
    Profiler* saved = current_profiler();
    set_current_profiler(nullptr);
    EigArgs g{};
    g.n = n;
    g.iu = iu;
    g.batch = 1;
    g.A = reinterpret_cast<double2*>(A);
    g.lda = n;
    g.strideA = n * n;
    g.X = reinterpret_cast<double2*>(Z);
    g.ldx = n;
    g.strideX = n * iu;
    g.w = w;
    g.ortol_rel = 1e-7;
    eig_bind_workspace(g, g_noalloc_ptr[dev]);
    int rc = eig_fp64(st, g);
    int fail = 0;
    if (rc == 0) {
        cudaError_t e = cudaMemcpyAsync(&fail, g.fail, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error(FORGE_ERR_CUDA, "zheevr_noalloc: %s", cudaGetErrorString(e));
            rc = FORGE_ERR_CUDA;
        }
    }
    set_current_profiler(saved);
    if (rc) return rc;
    return fail ? 1 : 0;
}
