// Launch interface between the host runtime (brx_api.cu, FP64 unit) and the
// mixed-precision unit (brx_mixed.cu). Plain host declarations only.
#pragma once
#include <cuda_runtime.h>
#include "brx_common.cuh"

namespace brx {

struct Launch {
    MeshDev mesh;
    StateDev state;
    BoundaryDev bnd;
    Work work;
    Ctrl *ctrl;
    int nscen, nslot, maxdeg;
    int grid_c, grid_f, grid_c256, grid_f256;
    cudaStream_t stream;
};

// Kernel kinds of one substep, in launch order within a stage.
enum KernelKind { K_DRAG = 0, K_BOUNDARY = 1, K_CELLS = 2, K_FACES = 3, K_GATHER = 4, K_LIMIT = 5, K_UPDATE = 6 };

// Mixed form (FP32 fluxes and updates, FP64 stage, pressure, bed source and
// mass): launch one kernel of the given kind for the given stage. Returns the
// number of kernels launched (0 for a boundary kernel without open faces).
int mixed_kernel(const Launch &L, int kind, int stage, double *rate_out);

}  // namespace brx
