// Types and device helpers shared by both arithmetic forms of the river step.
//
// One substep = drag(dt/2) -> 2 x [boundary -> cells -> faces -> gather ->
// limit -> update] -> control. Every kernel is batch-aware: cells and faces
// of many scenarios are packed into one index space, each element carries
// its scenario id, and each scenario owns a Ctrl block on the device that
// holds its clock (trial dt, elapsed time, hint) and its rejection status.
// The plain form is a batch of one.
//
// Restated from (file:line in the reference):
//   boundary     src/braids_core/sediment/river_exterior_bed.h:29-174,
//                src/braids_core/hydraulics/outlet_feasibility.py:25-38
//   cells        src/braids_support/gpu_fwave/reconstruction.cu:24-168 with the
//                wall_bed_hydraulics transforms (wall velocity bounds, LS
//                fallback, directional projection limiter)
//   faces        reconstruction.cu:170-212, resident_update.cu:11-148 with the
//                hydrostatic-reconstruction and reflecting-wall transforms,
//                augmented_fwave.cu:264-334
//   gather       src/braids_gpu/implicit_midpoint_fwave.cu:65-90,
//                src/braids_core/sediment/river_midpoint.h:21-29 (inventory),
//                river_explicit_boundary_budget.py:41-50 (reservation),
//                river_explicit.h:13-26 (CFL frequency)
//   limit        river_midpoint.h:30-41
//   update       river_midpoint.h:42-49, river_explicit.py:94-117
//   drag         river_hydraulic_drag.h:3-16, river_roughness.py:42-47
//   control      river_explicit.py:121-154
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include "brx_fwave.cuh"

namespace brx {

constexpr double EPS = 2.2204460492503131e-16;
constexpr double DBL_MIN_ = 2.2250738585072014e-308;

// Status bits of one stage. PRE bits are raised before the reference computes
// its CFL frequency, so a stage that raised one does not feed the step hint.
enum : unsigned {
    ST_SPATIAL = 1u,      // invalid state, boundary, reconstruction or face status
    ST_BUDGET = 2u,       // prescribed boundary exceeds the owner's stock
    ST_RATE = 4u,         // nonfinite rate
    ST_ENDPOINT = 8u,     // negative / nonfinite stage result
    ST_FREQ = 16u,        // nonfinite CFL frequency
    ST_TURBINE = 64u,     // rotor model outside its domain (the reference raises): the scenario fails
    ST_FATAL = 128u,      // an outlet section without an admissible solution (the reference raises ValueError)
    ST_PRE = ST_SPATIAL | ST_BUDGET | ST_RATE | ST_FREQ | ST_TURBINE | ST_FATAL,
};

// Record of one completed interval of a device-chained run
// (brx_advance_chain): the leading fields are brx_advance_stats' layout.
struct IvStat {
    int substeps, rejections, failed, pad;
    double min_dt, max_dt, cfl_max, hint;
    double ledger, gross;              // the interval's net inflow and gross boundary volume
};

// Per-scenario clock and controls, resident on the device.
struct Ctrl {
    // controls
    double grav, dry, cfl, speed_limit, roughness_value;
    int roughness_mode, active;       // active: scenario takes part in this interval
    // interval
    double dt_outer, time0, elapsed, hint, floor_, trial;
    int truncated, substeps, rejections, done;
    int failed, cur, max_substeps, one_stage;   // one_stage: a one-evaluation method (HLLC / Hancock)
    // this trial
    unsigned status1, status2;
    unsigned long long peak1, peak2;  // bit patterns of nonnegative doubles
    // diagnostics
    double min_dt, max_dt, cfl_max;
    double accepted_water_time;       // sum of accepted trial lengths (== elapsed)
    // water budget: each stage's sum over open faces of (outward water flux x
    // length) as the update uses it, and the interval's boundary ledger, the
    // net inflow volume of the accepted substeps (shoreline_solver.py:353-355);
    // bgross / gross: the same with |water x length| per face, an upper bound
    // of the reference's gross boundary volume sum_f |ledger_f| (the triangle
    // inequality), which scales its roundoff allowance
    double bflux[2], ledger;
    double bgross[2], gross;
    // FP32 copies for the mixed form's sweeps, refreshed with every trial
    float gravf, dryf, trialf, roughf;
    int cfl1, pad1;                         // stage 1 exceeded the CFL limit (mixed form, set after its gather)
    // device-chained intervals: how many follow this one, this one's index,
    // and where a completed interval is recorded (null outside a chain)
    int chain_left, chain_pos;
    IvStat *hist;
};

// Scenarios taking part in the current trial, packed: every sweep visits only
// their cells and faces, so a batch whose scenarios need different substep
// counts pays nothing for the ones that have finished their interval. The
// host sets it at the start of an interval; k_control rebuilds it after every
// trial (ascending scenario order).
struct ActiveDev {
    int *count;              // [0] runs, [1] cells, [2] faces
    int *cstart, *cdelta;    // (nscen+1), (nscen): per run, its first packed active cell index, and cell id - index
    int *fstart, *fdelta;    // the same for faces
    const int *cell_off, *face_off;   // (nscen+1) packed ranges of every scenario
};

// Position of packed index i in a prefix array: the largest j < n with start[j] <= i.
__device__ __forceinline__ int active_slot(const int *start, int n, int i)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Cell (face) id of the i-th active cell (face): runs of consecutive active
// scenarios are contiguous id ranges, so the map is i + delta of i's run (a
// fully active batch is one run: the identity).
__device__ __forceinline__ int active_cell(const ActiveDev &a, int i)
{
    return i + a.cdelta[active_slot(a.cstart, a.count[0], i)];
}

__device__ __forceinline__ int active_face(const ActiveDev &a, int i)
{
    return i + a.fdelta[active_slot(a.fstart, a.count[0], i)];
}

// Grid-stride sweep over the cells (faces) of the active scenarios; the body
// sees the packed id as `c` (`f`) and may `continue`.
#define FOR_ACTIVE_CELLS(A, c)                                                                              \
    for (int i_ = blockIdx.x * blockDim.x + threadIdx.x, n_ = (A).count[1]; i_ < n_; i_ += gridDim.x * blockDim.x) \
        if (const int c = active_cell((A), i_); true)
#define FOR_ACTIVE_FACES(A, f)                                                                              \
    for (int i_ = blockIdx.x * blockDim.x + threadIdx.x, n_ = (A).count[2]; i_ < n_; i_ += gridDim.x * blockDim.x) \
        if (const int f = active_face((A), i_); true)

struct MeshDev {
    int nc, nf, nadj, nscen;
    const int *owner, *neighbour, *bid, *offset, *faces, *signs;
    const int *bslot;        // per face: boundary slot (open faces) or -1
    const int *bmode;        // per face: hydraulic mode of its open segment, else 0
    const int *cell_sid, *face_sid;
    const int *cflags;       // per cell: bit0 owns an open face
    const double *normal, *length, *area;
    const double *ls_matrix, *ls_weight, *ls_delta;
    const double *disp, *disp_unit, *disp_len, *distance;
    ActiveDev act;           // scenarios of the current trial
};

// Rotor arrays on the device: the actuator sink and its diagnostics, and the
// balanced-pressure / ambient-stress face terms of scenarios that have rotors.
struct TurbDev {
    int nr, np, nucell;
    const int *hkt;             // (nscen) 1: the scenario has a rotor array
    const int *stress;          // (nscen) 1: its ambient viscosity is positive
    const int *rotor_sid;       // (nr)
    const int *support_offset, *support_cell;       // (nr+1), (ns)
    const double *support_weight, *support_density; // (ns)
    const int *plane_offset, *plane_cell;           // (nr+1), (np)
    const double *plane_delta;                      // (2, np)
    const double *param;                            // (nr, 8)
    const int *curve;                               // (nr, 4): thrust first, count; power first, count
    const double *curve_x, *curve_y;
    const double *curve_slope;                      // (y[k+1]-y[k])/(x[k+1]-x[k]) of each table knot
    const int *flat_thrust;                         // (nr) 1: the rotor's thrust table is constant
    const int *ucell, *uoff, *uent;                 // support cells of two or more entries -> their entries, rotor order
    const unsigned char *single;                    // (ns) 1: the entry's cell is in no other support entry
    const unsigned char *foot;                      // (nc) 1: a support cell (its actuator sink may be nonzero)
    const double *dxdy, *inverse, *xy, *mdisp, *nu; // (2,nadj) (3,nc) (2,nc) (4,nf) (nc)
    double *grad;               // (8, nc) wet gradients: u, v, eta, b (x, y)
    double *kcell;              // (ns) sink coefficient
    double *raw;                // (2, nc) actuator momentum sink
    double *trace;              // (10, nf) hydrostatically reconstructed face traces
    double *pface, *sface;      // (2, nf) pressure correction, ambient stress
    double *diag;               // (nr, 16) rotor diagnostics of the last sampled state
    int balanced;               // 1: balanced-pressure face term (f-wave owner); 0: HLLC owner
};

struct BoundaryDev {
    int nseg, nslot, nown;
    const int *scen_seg;     // (nscen+1) segment range per scenario
    const int *scen_own;     // (nscen+1) unique-owner range per scenario
    const int *seg_off;      // (nseg+1) slot range per segment
    const int *slot_face;    // (nslot)
    const int *seg_mode, *stage_policy;
    const double *ext_bed;   // (nslot)
    double *forcing;         // (2,nseg) sampled per stage
    int table_len;
    const double *table_time;   // (table_len)
    const double *table_value;  // (2, nseg, table_len)
    const int *own_cell, *own_off, *own_slot;  // unique owners, CSR into slots (boundary order)
    double *terms;           // (3, nslot) scratch: stage terms and weights
    double *trace, *flux;    // (3, nslot) each
    double *seg_sums;        // (3, nseg): wetted stage sum, wetted width, weight total
    const int *rt_off;       // (nseg+1) Q-H rating knots per mode-11 segment
    const double *rt_q, *rt_eta;
    const int *scen_chain;   // (nscen+1) normal-depth outlet chains per scenario
    const int *chain_off, *chain_slot;   // (nchain+1), slots in section order
    const double *chain_slope;           // (nchain)
    const double *weir;      // (3, nseg) free-weir crest, coefficient, effective width
    int *branch;             // (nslot) section-solve scratch: face branch
    double *invariant;       // (nslot) section-solve scratch: outgoing invariant / normal speed
    const int *crit_seg_chain;           // (nseg+1) critical-outlet chains per segment, or null
    const int *crit_chain_off, *crit_chain_slot;
    int *gslot, *gend;       // (nslot) wet-group scratch of the critical outlets
    int inlet;               // a mode-9 (exact-discharge inlet) segment exists
    const int *line_kind;    // (nseg) mode-9 reference line: 0 forcing stage, 1 critical, 2 normal; or null
    const double *line_slope;            // (nseg) energy slope of the normal lines
    const int *line_left, *line_right;   // (nslot) physical neighbour slots along the section, -1 none
    double *line_q, *line_stage;         // (nseg) solved line and its discharge (NaN: none)
};

// Accepted / stage state buffers.
struct StateDev {
    double *q[2];            // (3,nc) ping-pong: ctrl.cur holds the accepted state
    double *work;            // (3,nc) base after the opening drag
    double *q1;              // (3,nc) first-stage result
    const double *z;         // (nc) bed
};

// 128-byte cell record written by the cell kernel, read by the face kernel.
struct __align__(16) CellRec {
    double h, eta, u, v, b;
    double gx[4], gy[4];
    int flags, pad;          // bit0 flatten (hydro_constant), bit1 active
    double pad2;
};
static_assert(sizeof(CellRec) == 128, "cell record is one 128-byte line");

// Conservative wet-bank viscosity (shoreline_viscosity.py:46-72) of the
// scenarios with a positive coefficient: the flow engines' least-squares
// metric, cell centres, and the stage's velocity gradients and face stresses.
struct ViscDev {
    const double *nu;        // (nscen) coefficient [m2/s]; null: no scenario has one
    const double *dxdy;      // (2, nadj) centre offsets per CSR entry
    const double *inverse;   // (3, nc) least-squares pseudo-inverse
    const double *xy;        // (2, nc)
    double *grad;            // (4, nc) u_x, u_y, v_x, v_y of the safe state
    double *face;            // (2, nf) shared-face stress
};

struct Work {
    ViscDev visc;
    CellRec *rec;            // (nc)
    double2 *ws;             // (nf) water, CFL speed
    double4_32a *gf;             // (nf) pressure-deviation momentum flux: left x,y, right x,y
    double4_32a *lim;            // (nf) limited water, momentum correction x,y
    double *rate;            // (3,nc)
    double *theta;           // (nc)
};

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *addr, double v)
{
    // nonnegative doubles (including +inf) order like their bit patterns
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Warp-aggregated max of nonnegative doubles into ctrl[sid].peak: lanes with
// the same scenario reduce the high then the low 32 bits of their bit
// patterns (nonnegative doubles order like their bits) and the first lane of
// each group issues one atomic. Max is exact and order-free. Every lane of
// the warp must call it; lanes without a value pass valid = false.
__device__ __forceinline__ void warp_max_peak(unsigned long long *peak_of_sid0, size_t stride_bytes, int sid,
                                              bool valid, double v)
{
    const unsigned long long bits = valid ? (unsigned long long)__double_as_longlong(v) : 0ull;
    const unsigned same = __match_any_sync(0xffffffffu, valid ? sid : -1);
    const unsigned hi = (unsigned)(bits >> 32), lo = (unsigned)(bits & 0xffffffffull);
    const unsigned mhi = __reduce_max_sync(same, hi);
    const unsigned mlo = __reduce_max_sync(same, hi == mhi ? lo : 0u);
    if (valid && (int)(threadIdx.x & 31) == __ffs(same) - 1) {
        unsigned long long *addr = (unsigned long long *)((char *)peak_of_sid0 + stride_bytes * (size_t)sid);
        atomicMax(addr, ((unsigned long long)mhi << 32) | mlo);
    }
}

__host__ __device__ __forceinline__ double bits_to_double(unsigned long long b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
#endif
}

// Stage 2 and the trailing kernels skip a scenario whose first stage failed.
__device__ __forceinline__ bool stage1_failed(const Ctrl &c)
{
    if (c.status1) return true;
    const double f = bits_to_double(c.peak1);
    return c.trial * f > c.cfl * (1 + 1e-12);
}

__device__ __forceinline__ bool skip_stage(const Ctrl &c, int stage)
{
    if (!c.active || c.done) return true;
    return stage == 2 && stage1_failed(c);
}

__device__ __forceinline__ void raise_status(Ctrl &c, int stage, unsigned bits)
{
    atomicOr(stage == 1 ? &c.status1 : &c.status2, bits);
}

// Face traces of the hydrostatically reconstructed states for the rotor
// pressure correction (river_turbine_flow.h:39-52): surfaces, normal
// velocities and speeds of both sides, the common bed, constant flags.
__device__ __forceinline__ void put_trace(double *tr, int nf, int f, const double loc[8], bool cl, bool cr)
{
    const double hl = loc[0], hr = loc[4];
    tr[f] = hl + loc[3]; tr[nf + f] = hr + loc[7];
    tr[2 * nf + f] = hl > 0. ? loc[1] / hl : 0.; tr[3 * nf + f] = hr > 0. ? loc[5] / hr : 0.;
    tr[4 * nf + f] = hl > 0. ? hypot(loc[1], loc[2]) / hl : 0.;
    tr[5 * nf + f] = hr > 0. ? hypot(loc[5], loc[6]) / hr : 0.;
    tr[6 * nf + f] = loc[3]; tr[7 * nf + f] = loc[7];
    tr[8 * nf + f] = cl ? 1. : 0.; tr[9 * nf + f] = cr ? 1. : 0.;
}

// Momentum terms of a rotor array, in the reference's add_momentum order
// (river_turbine_flow.py:230-239): ambient stress, actuator sink, balanced
// pressure; face terms gathered as sum(s len flux) / area
// (flow2dh_fixed_bed_kernels.h:54-60 with unit depth weights). The HLLC
// owner's rotor hook has no balanced pressure (river_turbines.py:27-36):
// balanced = false.
__device__ __forceinline__ void add_rotor_momentum(const MeshDev &m, const TurbDev &t, int sid, int c, double area,
                                                   double &r1, double &r2, bool balanced = true)
{
    const int nc = m.nc, nf = m.nf;
    if (t.stress[sid]) {
        double x = 0., y = 0.;
        for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
            const int f = m.faces[k];
            x += m.signs[k] * m.length[f] * t.sface[f];
            y += m.signs[k] * m.length[f] * t.sface[nf + f];
        }
        r1 += 1. * x / area; r2 += 1. * y / area;
    }
    r1 += t.raw[c]; r2 += t.raw[nc + c];
    if (!balanced) return;
    double x = 0., y = 0.;
    for (int k = m.offset[c]; k < m.offset[c + 1]; ++k) {
        const int f = m.faces[k];
        x += m.signs[k] * m.length[f] * t.pface[f];
        y += m.signs[k] * m.length[f] * t.pface[nf + f];
    }
    r1 += 1. * x / area; r2 += 1. * y / area;
}

constexpr int BOUNDARY_TILES = 1024;   // tile slots of 64 faces per scenario (checked at set-up)
constexpr int MAX_CELL_FACES = 32;     // faces of one cell, checked at set-up

}  // namespace brx
