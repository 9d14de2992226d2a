// Launch interface between the host runtime (brx_api.cu, FP64 unit) and the
// mixed-precision unit (brx_mixed.cu). Plain host declarations only.
#pragma once
#include <cuda_runtime.h>
#include "brx_common.cuh"

namespace brx {

// FP32 geometry of the mixed form, packed for the sweep that reads it.
struct MixedGeo {
    const float4 *cinv;      // (nc) inverse LS normal matrix (i11, i12, i22, 0); zero when no gradient
    const int2 *cidx;        // (nadj) other cell (-1 none), flags: bit0 open face, bit1 stage outlet, bit2 wall
    const float4 *cent;      // (nadj) ls_delta x, y, this side's face displacement x, y
    const float *cwt;        // (nadj) least-squares weight
    const double *cw8;       // (nadj) signed length / area (mass bookkeeping)
    const float2 *fnorm;     // (nf) unit normal
    const float4 *fdisp;     // (nf) displacement owner side x, y, neighbour side x, y
    const float2 *fdist;     // (nf) |(mid - xy_owner).n|, |(xy_neighbour - mid).n|
};

struct Launch {
    MeshDev mesh;
    StateDev state;
    BoundaryDev bnd;
    Work work;
    Ctrl *ctrl;
    int nscen, nslot, maxdeg;
    int grid_c, grid_f, grid_c256, grid_f256;
    cudaStream_t stream;
    MixedGeo mx;
};

// Kernel kinds of one substep, in launch order within a stage.
enum KernelKind { K_DRAG = 0, K_BOUNDARY = 1, K_CELLS = 2, K_FACES = 3, K_GATHER = 4, K_LIMIT = 5, K_UPDATE = 6 };

// Mixed form (FP32 fluxes and updates, FP64 stage, pressure, bed source and
// mass): launch one kernel of the given kind for the given stage. Returns the
// number of kernels launched (0 for a boundary kernel without open faces).
int mixed_kernel(const Launch &L, int kind, int stage, double *rate_out);

}  // namespace brx
