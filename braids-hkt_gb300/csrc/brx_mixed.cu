// Mixed-precision form of the river step: the same kernels as the FP64 unit,
// instantiated with F = float. Riemann solves, reconstruction gradients,
// limiter and projection, advective fluxes and drag run in FP32; depth,
// stage (eta = h + b), hydrostatic pressures, the bed source, the mass
// update and the boundary sums stay FP64. This unit is compiled with FMA
// contraction and fast FP32 division / square root.
#define BRX_NS brx_mix
#include "brx_kernels.cuh"
#include "brx_launch.h"

namespace brx {

int mixed_kernel(const Launch &L, int kind, int stage, double *rate_out)
{
    cudaStream_t st = L.stream;
    switch (kind) {
    case K_DRAG:
        brx_mix::k_open_drag<float><<<L.grid_c256, 256, 0, st>>>(L.mesh, L.state, L.ctrl);
        return 1;
    case K_BOUNDARY:
        if (!L.nslot) return 0;
        brx_mix::k_boundary<float><<<L.nscen, 256, 0, st>>>(L.mesh, L.state, L.bnd, L.ctrl, stage);
        return 1;
    case K_CELLS:
        if (L.maxdeg <= 4)
            brx_mix::k_cells<float, 4><<<L.grid_c, 128, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, stage);
        else
            brx_mix::k_cells<float, MAX_CELL_FACES><<<L.grid_c, 128, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, stage);
        return 1;
    case K_FACES:
        brx_mix::k_faces<float><<<L.grid_f, 128, 0, st>>>(L.mesh, L.state, L.bnd, L.ctrl, L.work, stage);
        return 1;
    case K_GATHER:
        brx_mix::k_gather<<<L.grid_c256, 256, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, stage);
        return 1;
    case K_LIMIT:
        brx_mix::k_limit<<<L.grid_f256, 256, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, stage);
        return 1;
    case K_UPDATE:
        brx_mix::k_update<float><<<L.grid_c256, 256, 0, st>>>(L.mesh, L.state, L.ctrl, L.work, stage, rate_out);
        return 1;
    }
    return 0;
}

}  // namespace brx
