// Mixed-precision eigen-solver entry (filled in by the tensor-core path).
#include "eig.cuh"

namespace forge {

size_t eig_mixed_workspace_bytes(int64_t, int64_t, int64_t) { return 0; }

int eig_mixed(cudaStream_t, EigArgs&, void*) {
    set_error(FORGE_ERR_ARG, "mixed-precision eigen-solver is not available in this build");
    return FORGE_ERR_ARG;
}

}  // namespace forge
