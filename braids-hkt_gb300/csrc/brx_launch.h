// Launch interface between the host runtime (brx_api.cu, FP64 unit) and the
// mixed-precision unit (brx_mixed.cu). Plain host declarations only.
#pragma once
#include <cuda_runtime.h>
#include "brx_common.cuh"

namespace brx {

// FP32 geometry and tables of the mixed form, packed for the sweep that reads them.
struct MixedGeo {
    const float4 *cinv;      // (nc) inverse LS normal matrix (i11, i12, i22, 0); zero when no gradient
    const int2 *cidx;        // (nadj) other cell (-1 none), flags: bit0 open face, bit1 stage outlet, bit2 wall,
                             //   bit3 exterior-owner face (boundary slot), bit4 this cell owns the face
    const float4 *cent;      // (nadj) LS weight * ls_delta x, y; this side's face displacement x, y
    const float *cw4;        // (nadj) signed length / area, FP32 (momentum, outflow and CFL sums)
    const double *cw8;       // (nadj) signed length / area, FP64 (mass)
    const int *ccls;         // (nc) bit0: the cell has a stage outlet face
    const float2 *fnorm;     // (nf) unit normal
    const float4 *fdisp;     // (nf) displacement owner side x, y, neighbour side x, y
    const float2 *fdist;     // (nf) |(mid - xy_owner).n|, |(xy_neighbour - mid).n|
    // bed-derived tables, rebuilt from the FP64 bed by K_BED
    float *cdb;              // (nadj) bed of the other cell - own bed (0 without one)
    float *fdb;              // (nf) neighbour bed - owner bed
    float2 *gbed;            // (nc) limited bed gradient
    // FP32 primitives of the two stage inputs (32 bytes per cell each)
    float4 *prim[2];
    // rotor arrays: FP32 flow metric and face terms
    const float2 *hdxy;      // (nadj) centre offsets of the flow least-squares metric
    const float4 *hmd;       // (nf) face-midpoint displacement: owner x, y; neighbour x, y
    const float2 *hcc;       // (nf) neighbour centroid - owner centroid
    float *hgrad;            // (6, nc) wet gradients of u, v, eta
    float2 *hp, *hs;         // (nf) balanced-pressure correction, ambient stress
    // HLLC / MUSCL-Hancock method (its own incidence, faces ascending per cell)
    const int2 *hent;        // (nadj) face or ~face (neighbour side); other cell, -1 wall, -2 open face
    const float4 *hgeo;      // (nadj) LS offset over its squared length (x, y); face midpoint - centroid (x, y)
    const float4 *hinv;      // (nc) least-squares inverse (i11, i12, i22, 0)
    const float *hw4;        // (nadj) signed length / area, FP32 (momentum, outflow and CFL sums)
    const double *hw8;       // (nadj) signed length / area, FP64 (mass)
    float *hcdb;             // (nadj) bed of the other cell - own bed (0 for walls and open faces)
};

// Cell tiles of the mixed f-wave stage sweep (km_tile): consecutive cells of
// one scenario, with the ring of neighbours whose records the tile's faces
// need (ring 1) and the ring their records read (ring 2). A tile's local
// slots: [0, T) its cells, then ring 1, then ring 2.
struct TileDev {
    int ntiles, cells;       // tiles, cells per tile (the last tile of a scenario may be shorter)
    int cap_prims, cap_recs, cap_faces;   // shared-memory slots: max over tiles
    const int4 *info;        // (ntiles) first cell, end cell, start in halo, start in face list
    const int4 *info2;       // (ntiles) ring-1 cells, ring-2 cells, faces, start of the ring-1 entries (x4)
    const int *halo;         // ring-1 then ring-2 cell ids of each tile
    const int2 *tent;        // (nadj) entries of each cell in its own tile: neighbour's local slot (-1 none), flags
    const int2 *hent;        // (4 per ring-1 cell) the same for the ring-1 cells of each tile
    const int *tfslot;       // (nadj) the face-list slot of each entry in its cell's tile
    const int4 *tface;       // face lists: face, owner's local slot, neighbour's local slot (-1 none), 0
};
// HLLC kinds of one substep (their launch-shape slots), shared by both forms.
enum HllcKind { KH_CELLS = 20, KH_PREDICT = 21, KH_BOUNDARY = 22, KH_FACES = 23, KH_BUDGET = 24, KH_TURB = 25,
                KH_UPDATE = 26, KH_TURB0 = 27 };

// Launch shape of one kernel kind: threads per block and the grid cap in
// resident blocks per SM (grid = min(ceil(n / block), per_sm * SMs); the
// sweeps are grid-stride loops, so any shape covers every element).
constexpr int NSHAPE = 32;
struct LaunchShape {
    int block, per_sm;
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
    TurbDev turb;            // rotor arrays (valid when has_turb)
    int has_turb;
    int sms;
    LaunchShape shape[NSHAPE];
    TileDev tiles;           // valid when tile_smem > 0
    int tile_smem;           // dynamic shared memory of the tile sweep (0: the separate sweeps)
};

inline int shape_grid(const Launch &L, int kind, int n)
{
    const LaunchShape &sh = L.shape[kind];
    const int g = (n + sh.block - 1) / sh.block, cap = sh.per_sm * L.sms;
    return g < 1 ? 1 : (g < cap ? g : cap);
}

// Kernel kinds of one substep, in launch order within a stage.
enum KernelKind { K_DRAG = 0, K_BOUNDARY = 1, K_CELLS = 2, K_FACES = 3, K_GATHER = 4, K_LIMIT = 5, K_UPDATE = 6 };
// Mixed form only: first-stage primitives of a state placed in work, the
// bed-derived tables, the limited water flux into a caller buffer.
enum MixedAux { K_PRIM = 8, K_BED = 9, K_WATER = 10, K_HKT_GRAD = 12, K_HKT_FACES = 13 };
// Rotor-array terms of one stage (both forms; FP64 kernels of the FP64 unit).
enum { K_TURB = 11 };
// Wet-bank viscosity of one stage (both forms; FP64 kernels of the FP64 unit).
enum { K_VISC = 14 };
// Mixed form: cells, faces and gather of one stage in one pass over cell
// tiles staged in shared memory (meshes of at most four faces per cell).
enum { K_TILE = 15 };
constexpr int TILE_THREADS = 256;
// Shared memory of the tile sweep for the given slot capacities, and its
// one-time attribute set-up (outside stream capture). Returns a CUDA error code.
int mixed_tile_smem(int cap_prims, int cap_recs, int cap_faces);
int mixed_tile_prepare(int smem_bytes);

// Mixed form (FP32 sweeps, FP64 stage pair, depth and mass): launch one kernel
// of the given kind for the given stage; out is the rate buffer of K_UPDATE or
// the water buffer of K_WATER. Returns the number of kernels launched (0 for a
// boundary kernel without open faces).
int mixed_kernel(const Launch &L, int kind, int stage, double *out);

// Largest block the mixed form's kernel of this kind accepts (its launch
// bounds and registers), 0 for a kind without a tunable kernel.
int mixed_max_block(int kind, int maxdeg);

// Mixed form of the HLLC / MUSCL-Hancock method: launch one kernel of the
// given HLLC kind (cells, predictor source, faces, budget, update; the
// boundary, drag and rotor kinds are the f-wave's). Returns launches.
int mixed_hllc_kernel(const Launch &L, int kind);

}  // namespace brx
