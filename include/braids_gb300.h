/*
 * braids_gb300.h - C ABI of the GB300 river solver step (BRAIDS-HKT
 * augmented f-wave path).
 *
 * Plain C types only: host pointers for set-up arrays, device pointers for
 * the resident state, sizes as int. Every call returns BRX_OK (0) or a
 * positive error code; brx_last_error() describes the last failure of the
 * calling thread. No call traps or aborts.
 *
 * Layouts follow the reference's component-major (C-contiguous SoA) records:
 * q is (3,nc) rows h, hu, hv; normal (2,nf); displacement (2,2,nf)
 * [component][side][face]; distance (2,nf); ls_matrix (4,nc); ls_delta
 * (2,nadj). Indices are zero-based int32 with -1 for "none".
 *
 * Batching: nscen scenarios are packed into one index space. cell_offset and
 * face_offset (nscen+1) give each scenario's cell and face range; all
 * indices (owner, neighbour, faces, boundary_faces) are global. bid[f] of an
 * open face is its global segment number; seg_offset (nscen+1) gives each
 * scenario's segment range. One scenario is the plain form.
 */
#ifndef BRAIDS_GB300_H
#define BRAIDS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define BRX_OK 0
#define BRX_ERR_ARGUMENT 1      /* invalid size, index or pointer */
#define BRX_ERR_CUDA 2          /* CUDA runtime failure */
#define BRX_ERR_STATE 3         /* call out of order (e.g. no state bound) */
#define BRX_ERR_REJECTED 4      /* trial rejected / interval could not be completed */
#define BRX_ERR_UNSUPPORTED 5   /* mesh or mode outside the supported scope */

/* Arithmetic forms. */
#define BRX_FP64 0    /* FP64 everywhere, reference operation order, no FMA */
#define BRX_MIXED 1   /* FP32 fluxes and updates; FP64 stage, bed source, mass */

/* Rejection causes reported per scenario (bit set). */
#define BRX_ST_SPATIAL 1u
#define BRX_ST_BUDGET 2u
#define BRX_ST_RATE 4u
#define BRX_ST_ENDPOINT 8u
#define BRX_ST_FREQ 16u
#define BRX_ST_CFL 32u      /* dt * max frequency above the CFL target */
#define BRX_ST_TURBINE 64u  /* rotor model outside its domain: the scenario fails (failed = 4) */

typedef struct brx_solver brx_solver;

/* Per-scenario outcome of one brx_advance call
 * (mirrors the diagnostics of RiverExplicit.advance,
 *  src/braids_core/sediment/river_explicit.py:150-154). */
typedef struct {
    int substeps;        /* accepted SSPRK(2,2) substeps */
    int rejections;      /* rejected trials */
    int failed;          /* 0 ok, 1 dt floor / rejection limit, 2 substep limit, 4 rotor model error */
    int pad;
    double min_dt, max_dt, accepted_cfl_max, hint;
} brx_advance_stats;

const char *brx_last_error(void);
int brx_version(void);

/* Create a solver resident on the current CUDA device. Replaces the records
 * dict of the reference's physics owner (river_mesh_records.initialize,
 * src/braids_core/sediment/adaptive_river_worker.py:228) and the geometry
 * upload of ResidentReconstruction / ResidentFlux
 * (src/braids_support/gpu_fwave/reconstruction.py:91-118). All arrays are
 * host memory and are copied. displacement_length (2,nf) is |displacement| per
 * face side; pass NULL to have it computed here with the C library's hypot
 * (pass the caller's own values when they must match another machine's
 * geometry records bit for bit). */
int brx_solver_create(int nscen, const int *cell_offset, const int *face_offset,
                      int nc, int nf, int nadj,
                      const int *owner, const int *neighbour, const int *bid,
                      const int *offset, const int *faces, const int *signs,
                      const double *normal, const double *length, const double *area,
                      const double *ls_matrix, const double *ls_weight, const double *ls_delta,
                      const double *displacement, const double *displacement_length,
                      const double *distance, int nseg, const int *seg_offset, const int *boundary_offset,
                      const int *boundary_faces, int precision, brx_solver **out);

int brx_solver_destroy(brx_solver *s);

/* Physical and numerical controls of one scenario (scen = -1: all).
 * Replaces the reference's Parameters / CurrentRiverControls
 * (src/braids_core/sediment/bend_methods_v1.py:64-83, current_river_solver.py:17-32)
 * and river_roughness.selected (river_roughness.py:23-38): roughness_mode 1
 * Chezy, 2 Manning, 3 White-Colebrook log layer, 4 classical. */
int brx_controls_set(brx_solver *s, int scen, double gravity, double dry, double cfl,
                     double speed_limit, int roughness_mode, double roughness_value);

/* Q-H rating curves of the mode-11 outlets (replaces RatingOutlet's tables,
 * src/braids_core/sediment/river_rating_outlet.py:10-18): segment s's knots
 * are offset[s] .. offset[s+1]-1 of discharge [m3/s] / elevation [m], the
 * elevations increasing; offset (nseg+1), host arrays, copied. Call before
 * brx_boundary_set when any segment has mode 11. */
int brx_rating_set(brx_solver *s, const int *offset, const double *discharge, const double *elevation);

/* Connected face chains of the normal-depth outlets (mode 10): chain c's
 * faces (global ids, in section order) are faces[offset[c] .. offset[c+1]-1],
 * its bed slope slope[c] (the reference's NormalOutlet sections,
 * src/braids_core/sediment/river_normal_outlet.py:16-27, ordered by
 * connected_opening_chains). Chains in scenario order. Host arrays, copied;
 * call before brx_boundary_set when any segment has mode 10. */
int brx_outlet_chains_set(brx_solver *s, int nchain, const int *offset, const int *faces, const double *slope);

/* Connected face chains of the critical outlets (mode 4): segment s's
 * chains are seg_chain[s] .. seg_chain[s+1]-1, chain c's faces (global ids,
 * section order) faces[offset[c] .. offset[c+1]-1] (CriticalOutlet's
 * chains, src/braids_core/sediment/river_exterior_outlet.py:20-21; the
 * opening is solved whole, then per wet group of each chain when a group
 * split occurs). Host arrays, copied; before brx_boundary_set. */
int brx_critical_chains_set(brx_solver *s, const int *seg_chain, const int *offset, const int *faces);

/* Free-weir outlets (mode 5): param (3, nseg) crest [m], coefficient
 * [m^0.5/s] and effective width [m] per segment (FreeWeir's parameters,
 * src/braids_core/sediment/river_exterior_outlet.py:73-79). Host array,
 * copied; call before brx_boundary_set when any segment has mode 5. */
int brx_weir_set(brx_solver *s, const double *param);

/* Reference water lines of the exact-discharge inlets (mode 9), per
 * segment kind: 0 the forcing stage (inlet.stage_discharge /
 * inlet.depth_discharge), 1 critical depth (inlet.critical_discharge:
 * Q^2 W / (g A^3) = 1 on the exterior face beds, minimum specific energy
 * among the wet-width branches; CriticalSection,
 * src/braids_core/sediment/river_exterior_section.py:10-41 and
 * river_exterior_section.h), 2 normal depth (inlet.normal_discharge: the
 * lowest level whose uniform flow at the energy slope carries Q, with the
 * solver's roughness law at the section radius and wetted steps between
 * neighbouring faces; NormalSection, river_exterior_normal.py:30-74 and
 * river_exterior_normal.h, without bedform feedback). slope (nseg) the energy
 * slope of kind-2 lines; left, right (nf) the physical neighbour face of each
 * face along its section or -1 (NormalSection's adjacency,
 * river_exterior_normal.py:11-27; the host helper
 * braids_hkt_gb300.mesh.section_neighbours). The line is solved before the
 * exterior flux of every stage (kept while the discharge is unchanged); a
 * section without a root rejects the trial. Host arrays, copied. */
int brx_inlet_lines_set(brx_solver *s, const int *kind, const double *slope, const int *left, const int *right);

/* Open-boundary set-up for all segments: hydraulic mode (2 stage, 3 free
 * outflow, 4 critical: outgoing characteristic discharge sqrt(g A^3 / B)
 * on the controlled faces, river_exterior_outlet.h; 5 free weir: the
 * common subcritical stage whose outgoing Lax-curve
 * discharge equals coefficient x width x head^1.5, river_exterior_outlet.h;
 * 6 total discharge; 9 exact discharge with a reference water line (the
 * forcing stage): boundary Riemann solutions against a virtual reservoir at
 * that line whose common normal velocity makes the net section discharge
 * exact, then the stock-aware inlet allocation, river_exterior_inlet.h and
 * src/braids_core/hydraulics/inlet_feasibility.py; 10 normal depth:
 * per face chain the level at which the outgoing characteristic discharge
 * equals the uniform-flow conveyance, river_normal_outlet.h; 11 Q-H rating
 * curve: one common water elevation at which the outgoing characteristic
 * discharge equals the curve, river_rating_outlet.h), stage reversal
 * policy, exterior bed per face (nf, read on open faces) and forcing (2,nseg)
 * rows discharge, stage. Replaces ExteriorBed construction
 * (src/braids_core/sediment/river_exterior_bed.py:47-93). */
int brx_boundary_set(brx_solver *s, const int *seg_mode, const int *stage_policy,
                     const double *exterior_bed, const double *forcing);

/* Replace the constant forcing of every open segment, host forcing (2, nseg)
 * in the layout of brx_boundary_set (row 0 discharge, row 1 stage), keeping
 * modes, exterior beds and section tables; solved inlet reference lines are
 * cleared. For serving loops that re-use a resident scenario slot for a
 * request with its own discharge (the reference sets a scenario's forcing
 * once, river_exterior_bed.py:189-235). Not while an asynchronous interval
 * is in flight. */
int brx_forcing_set(brx_solver *s, const double *forcing);

/* Piecewise-linear forcing tables: time (len >= 2, increasing), value
 * (2,nseg,len) rows discharge and stage. len = 0 returns to constant forcing.
 * Replaces RiverHydraulicSchedule.sample
 * (src/braids_core/river_hydraulic_schedule.py:57-65): the same knot choice
 * and (1 - w) y_i + w y_{i+1}. Outside the table the end values hold (the
 * reference raises instead; keep evaluation times inside the table). */
int brx_forcing_table_set(brx_solver *s, int len, const double *time, const double *value);

/* Bind caller-owned DEVICE buffers: q (3,nc) accepted state, updated in place;
 * z (nc) bed. The reference keeps q and z in its owner
 * (ShorelineSolver.q / .z, src/braids_core/sediment/shoreline_solver.py:275). */
int brx_state_bind(brx_solver *s, double *q_device, double *z_device);

/* Advance every active scenario over [time, time+dt] with the adaptive
 * SSPRK(2,2) controller. Replaces RiverExplicit.advance
 * (src/braids_core/sediment/river_explicit.py:121-154). stats: nscen entries
 * (host), may be NULL. Returns BRX_ERR_REJECTED if any scenario failed. */
int brx_advance(brx_solver *s, double dt, double time, brx_advance_stats *stats);

/* As brx_advance with one interval per scenario: scenario i advances over
 * [time[i], time[i] + dt[i]] (host arrays of nscen); dt[i] <= 0 leaves it
 * idle. Scenarios keep independent clocks inside the same launches. */
int brx_advance_batch(brx_solver *s, const double *dt, const double *time, brx_advance_stats *stats);

/* Mixed f-wave form, cells of at most four faces: run the cell, face and
 * gather sweeps of each stage as one pass over tiles of `cells` consecutive
 * cells of a scenario (0 = the separate sweeps, the default). Each block
 * stages its tile's primitives with two rings of neighbours in shared
 * memory, forms the records of the tile and of the first ring, the fluxes
 * of every face of the tile's cells and the tile's gathers there; records
 * and momentum fluxes no longer pass through device memory. The arithmetic
 * of every record, face and gather is the separate sweeps'. No reference
 * counterpart (its GPU path runs one kernel per sweep,
 * src/braids_support/gpu_fwave/resident_update.cu); the tile size is what
 * the autotuner picks. */
int brx_tile_set(brx_solver *s, int cells);
int brx_tile_get(const brx_solver *s, int *cells, int *smem_bytes);

/* Several consecutive intervals per scenario in one call: scenario i
 * advances over [t_k, t_k + dt[i]] for k = 0 .. intervals-1, with t_0 =
 * time[i] and t_{k+1} = t_k + dt[i] (the owner's outer loop of steps at a
 * fixed interval, src/braids_core/sediment/adaptive_river_worker.py:646-667,
 * without the host between the steps). A scenario that completes an
 * interval begins its next one on the device at once, so the batch does not
 * drain at every interval end. Each interval's substeps, state, controller
 * statistics and boundary ledger are those of `intervals` consecutive
 * brx_advance_batch calls with the same start times. stats (host, nscen x
 * intervals, scenario-major, may be NULL) as brx_advance; ledger and gross
 * (host, nscen x intervals, may be NULL) each interval's net inflow volume
 * and gross boundary volume as brx_ledger_get / brx_ledger_gross_get give
 * them after one interval (those getters then report the last interval).
 * An interval after a failed one reports failed = 3 (not run); intervals
 * is 1..65536. Returns BRX_ERR_REJECTED if any scenario failed. */
int brx_advance_chain(brx_solver *s, const double *dt, const double *time, int intervals,
                      brx_advance_stats *stats, double *ledger, double *gross);

/* One SSPRK(2,2) trial of exactly dt on every active scenario
 * (RiverExplicit._single, river_explicit.py:94-119). On acceptance the bound
 * state is replaced; status (nscen, host) gets the rejection bits (0 =
 * accepted) and peak (nscen, host) the larger stage CFL frequency. */
int brx_substep(brx_solver *s, double dt, double time, unsigned *status, double *peak);

/* One spatial residual of the bound state (RiverExplicit.rate with
 * interval base = state, river_explicit.py:63-92): rate (3,nc) and limited
 * water flux (nf) into caller DEVICE buffers; status/freq per scenario (host). */
int brx_rate(brx_solver *s, double dt, double time, double *rate_device, double *water_device,
             unsigned *status, double *freq);

/* Scenario mask for brx_advance / brx_substep / brx_rate (nscen ints, host;
 * nonzero = active). All scenarios are active after creation. */
int brx_scenarios_activate(brx_solver *s, const int *active);

/* Rotor arrays (replaces the reference's river_turbine_flow.install with a
 * ThetisArray, src/braids_core/sediment/river_turbine_flow.py:222-252 and
 * river_turbine_thetis.py:300-318). Called once, after brx_solver_create.
 *   rotor_scenario (nrotor)      owning scenario of each rotor
 *   param (nrotor, 8)            D, hub elevation, minimum bed clearance,
 *                                minimum surface clearance, gate tolerance,
 *                                control mode (0 constant Ct, 1 speed table,
 *                                2 incident-speed table, 3 incident-speed
 *                                curves), Ct and Cp of the constant mode
 *   curve (nrotor, 4)            first index and count of the thrust (Ct) and
 *                                power (Cp) tables in curve_x / curve_y
 *   support_offset (nrotor+1), support_cell, support_weight, support_density
 *                                footprint cells (global ids), normalized bump
 *                                weights, bump density integrals
 *   plane_offset (nrotor+1), plane_cell, plane_delta (2, np)
 *                                rotor-plane crossings and their displacement
 *                                from the cell centroid
 *   dxdy (2, nadj), inverse (3, nc), xy (2, nc), mid_disp (4, nf)
 *                                the flow engines' least-squares metric
 *                                (bend_methods_v1.py:100-128)
 *   nu (nc)                      ambient eddy viscosity
 *   hkt (nscen)                  1 where the scenario has a rotor array
 * All arrays are host memory, copied. */
int brx_turbines_set(brx_solver *s, int nrotor, const int *rotor_scenario, const double *param,
                     const int *curve, int ncurve, const double *curve_x, const double *curve_y,
                     const int *support_offset, const int *support_cell, const double *support_weight,
                     const double *support_density, const int *plane_offset, const int *plane_cell,
                     const double *plane_delta, const double *dxdy, const double *inverse, const double *xy,
                     const double *mid_disp, const double *nu, const int *hkt);

/* Rotor diagnostics (nrotor, 16 doubles, host) of the bound state
 * (hkt_diagnose: river_turbine_flow.py:240-241): active, inactive reason,
 * coverage margin, bed clearance, local speed, upstream speed, mean depth,
 * Ct, Cp, force/rho [m4/s2], useful power/rho [m5/s3], removed power/rho,
 * lowest rotor-plane surface, highest bed, error code, reserved. */
int brx_turbines_diagnose(brx_solver *s, double *out);
/* The same record for the state of the last evaluated stage. */
int brx_turbines_last(brx_solver *s, double *out);

/* Exner bed model (replaces ShorelinePhysics.finish with morphology:
 * src/braids_core/sediment/shoreline_solver.py:218-240 with the MPM
 * capacity of river_mpm.py:21-33, one grain size, no secondary-flow spiral).
 *   enabled (nscen)          1 where a scenario has a bed model
 *   param (nscen, 5)         grain diameter [m], porosity, Chezy coefficient,
 *                            morphological factor, sediment working depth [m]
 *   bedbc (nf)               boundary faces: 0 wall, 1 prescribed feed, 2 open
 *                            outflow, 3 transport capacity
 *   feed (nf), rock (nc)     prescribed solid volume inflow per length [m2/s],
 *                            non-erodible elevation
 *   dxdy, inverse, xy        the flow engines' least-squares metric (as for
 *                            brx_turbines_set) and the cell centroids
 * Host arrays, copied. */
int brx_exner_set(brx_solver *s, const int *enabled, const double *param, const int *bedbc, const double *feed,
                  const double *rock, const double *dxdy, const double *inverse, const double *xy);

/* One bed update of the bound accepted state over dt (nscen, host; 0 skips a
 * scenario) times each scenario's morphological factor. The bound bed is
 * replaced where the scenario's checks pass (finite, above the non-erodible
 * layer, solid-volume residual <= 1e-10 m3, change <= 5% of the depth);
 * stats (nscen, 8 doubles, host): ok, residual, boundary solid volume, donor
 * minimum, maximum relative change, slope-operator failure. */
int brx_exner(brx_solver *s, const double *dt, double *stats);

/* Asynchronous form of brx_advance_batch for serving loops: start launches
 * the interval's first CUDA-graph chunk and returns; poll never blocks. It
 * sets *done = 0 while the interval runs (launching the next chunk when the
 * last one has finished) and *done = 1 once every scenario has completed,
 * with stats (nscen) filled and the return code of brx_advance_batch. One
 * interval per solver at a time; solvers on their own streams overlap. */
int brx_advance_start(brx_solver *s, const double *dt, const double *time);
int brx_advance_poll(brx_solver *s, int *done, brx_advance_stats *stats);

/* Compensated totals of the bound state per scenario (out: nscen x 2, host):
 * water volume sum(A h) [m3] and mechanical energy per unit density
 * sum(A (|hu|^2 / 2h + g h^2 / 2 + g h z)) [m5/s2], Neumaier-summed in a fixed
 * order (the same value on every run). The reference checks its water budget
 * on the host (shoreline_solver.py:345-372); this gives the device-resident
 * batch the same totals without copying the state. */
int brx_totals(brx_solver *s, double *out);

/* Device bytes the solver holds (for admission against a memory budget). */
long long brx_solver_bytes(const brx_solver *s);

/* Hydraulic methods. */
#define BRX_METHOD_FWAVE 0   /* augmented f-wave, SSPRK(2,2) (RiverExplicit) */
#define BRX_METHOD_HLLC 1    /* HLLC / HLLE MUSCL-Hancock (RiverHLLC, FP64 form only) */

/* The HLLC operator's own stencil (replaces HLLCHydraulics.__init__,
 * src/braids_core/hydraulics/hllc.py:16-61). Per CSR entry k of the cell
 * incidence (the offsets of brx_solver_create; each cell's faces in
 * ascending face number, hllc.py:29-34):
 *   entry_face (nadj)    face id, or its bitwise NOT where the cell is the
 *                        face's neighbour
 *   entry_other (nadj)   the other cell, -1 for a wall, -2 for an open face
 *   entry_geo (4, nadj)  offset to the other centroid (wall: the mirror
 *                        2 ((mid - xy) . n) n) x, y; face midpoint minus the
 *                        cell centroid x, y
 *   inverse (3, nc)      pinv of sum d d^T / |d|^2 over neighbours and walls
 *                        (open faces excluded): i11, i12, i22
 * Host arrays, copied. */
int brx_hllc_set(brx_solver *s, const int *entry_face, const int *entry_other, const double *entry_geo,
                 const double *inverse);

/* Conservative wet-bank viscosity of each scenario (replaces the reference's
 * shoreline_viscosity.install, src/braids_core/sediment/shoreline_viscosity.py:
 * 46-72, whose add_momentum hook it computes every spatial evaluation after
 * the rotor terms): nu (nscen) coefficient [m2/s], 0 for none; the flow
 * engines' least-squares metric of the packed mesh (bend_methods_v1.py:
 * 100-128): dxdy (2, nadj) centre offsets per CSR entry, inverse (3, nc)
 * pseudo-inverse (i11, i12, i22), and cell centres xy (2, nc). The f-wave
 * method only (BRX_ERR_UNSUPPORTED with HLLC). Both arithmetic forms. */
int brx_viscosity_set(brx_solver *s, const double *nu, const double *dxdy, const double *inverse, const double *xy);

/* Select the hydraulic method advanced by brx_advance / brx_advance_batch /
 * brx_advance_start / brx_substep (replaces the reference's river_hllc.install,
 * src/braids_core/hydraulics/river_hllc.py:95-101). BRX_METHOD_HLLC needs
 * the FP64 form and brx_hllc_set; brx_rate stays an f-wave residual. */
int brx_method_set(brx_solver *s, int method);

/* The forcing of the last evaluated stage, host out (2, nseg): rows
 * discharge and stage as the exterior flux used them (the sampled tables;
 * for the critical / normal inlet lines the solved reference line), as the
 * reference's ExteriorBed.forcing after evaluate. */
int brx_forcing_get(brx_solver *s, double *out);

/* Boundary ledger of the last interval, host out (nscen): the net volume
 * [m3] that entered through open faces over the accepted substeps,
 * -sum_k dt_k sum_f water_f length_f with each stage's water as the update
 * used it (SSPRK: the mean of the two stages; HLLC: its one evaluation). The
 * owner's water budget (ShorelineSolver.step, shoreline_solver.py:353-360)
 * compares it with the volume change (brx_totals before and after). */
int brx_ledger_get(brx_solver *s, double *out);

/* Gross boundary volume of the last interval, host out (nscen): the sum over
 * the accepted substeps of dt_k sum_f |water_f length_f| (SSPRK: the mean of
 * the two stages' sums). It bounds the reference's gross volume
 * sum_f |ledger_f| from above and scales the owner's FP64 roundoff allowance
 * (water_increment_roundoff_limit, shoreline_solver.py:29-39, 356-357). */
int brx_ledger_gross_get(brx_solver *s, double *out);

/* Step hint carried between brx_advance calls (nscen, host; <= 0 = none). */
int brx_hint_get(brx_solver *s, double *hint);
int brx_hint_set(brx_solver *s, const double *hint);

/* Number of substeps captured per CUDA graph replay inside brx_advance. */
int brx_graph_chunk_set(brx_solver *s, int substeps);

/* Launch shape of one kernel kind (the kinds of brx_profile_substep: 0 drag,
 * 2 cells, 3 faces, 4 gather, 5 limit, 6 update, 12 / 13 rotor gradients /
 * face terms, 15 the mixed tile sweep (block fixed at 256, one tile per block
 * and grid-stride step); HLLC 20 cells, 21 predictor, 23 faces, 24 budget,
 * 26 update):
 * threads per block (a multiple of 32 up to the kernel's limit) and the grid
 * cap in blocks per SM. Every sweep is a grid-stride loop, so results do not
 * depend on the shape. The autotuner (braids_hkt_gb300.autotune) sets these;
 * no counterpart in the reference. get also returns the kernel's limit. */
int brx_launch_shape_set(brx_solver *s, int kind, int block, int blocks_per_sm);
int brx_launch_shape_get(brx_solver *s, int kind, int *block, int *blocks_per_sm, int *max_threads);

/* Time one SSPRK(2,2) trial of exactly dt kernel by kernel with CUDA events
 * on the solver stream (no graph). ms (cap entries) gets each launch's
 * duration and kind (cap entries) its kernel: 0 drag, 1 boundary, 2 cells,
 * 3 faces, 4 gather, 5 limit, 6 update, 7 control, 11 rotor terms (four
 * kernels timed together); for BRX_METHOD_HLLC 20 cells, 21 predictor
 * source, 22 boundary, 23 faces, 24 budget, 25 rotor terms at the predicted
 * state, 26 update, 27 rotor terms at the start state. *count gets the number
 * of launches. The bound state is advanced as by brx_substep. */
int brx_profile_substep(brx_solver *s, double dt, double time, int cap, double *ms, int *kind, int *count);

/* FMA throughput of the current device (no counterpart in the reference):
 * precision 0 FP64, 1 FP32. Eight independent FMA chains per thread at full
 * occupancy, timed with CUDA events (best of five launches after one warm-
 * up). tflops gets 2 x FMAs / s / 1e12, ms (may be NULL) the launch time. It
 * is the compute roofline of the FP64 form and of the mixed form's FP32
 * sweeps. */
int brx_fma_rate(int precision, double *tflops, double *ms);

/* Allocation-free spatial residual of one closed scenario (walls only, no
 * open boundaries). It has no counterpart in the reference: it exists for
 * callers that may not allocate device memory once running - hosts that hand
 * out a fixed device-memory budget at start-up, or real-time loops where a
 * cudaMalloc would synchronise the device - and computes what brx_rate
 * computes (rate (3,nc), limited water flux (nf), status bits and CFL
 * frequency) without a solver handle and without allocating.
 *
 * Every mesh, state and output pointer is the caller's DEVICE memory, laid
 * out as for brx_solver_create and brx_rate; status and freq are host
 * pointers (may be NULL). At most 16384 cells and 32768 faces: larger meshes
 * get BRX_ERR_UNSUPPORTED. The stage scratch is one static device array of
 * about 7.4 MB that every GPU loading this library holds until process exit.
 * The first call in each CUDA context (each device's primary context, and
 * again after a cudaDeviceReset, which loads the module anew) looks up that
 * array's device address (cudaGetSymbolAddress) with the device current;
 * make that first call before any stream capture. Calls share the array and
 * rewrite what they read, so consecutive calls are independent, but calls
 * that overlap on the GPU (other streams, other host threads) race on it.
 * The call runs on `stream` (cudaStream_t as void*, NULL for the default
 * stream) and returns after it has finished. Invalid device topology (index
 * out of range, a cell with more than 32 faces) is detected on the device
 * and reported as BRX_ERR_ARGUMENT with the spatial status bit, without
 * touching the mesh further; on any nonzero return rate and water are not
 * written. */
int brx_rate_noalloc(int nc, int nf, int nadj, const int *owner, const int *neighbour, const int *offset,
                     const int *faces, const int *signs, const double *normal, const double *length,
                     const double *area, const double *ls_matrix, const double *ls_weight, const double *ls_delta,
                     const double *displacement, const double *displacement_length, const double *distance,
                     const double *q, const double *z, double gravity, double dry, double cfl, double dt,
                     double *rate, double *water, unsigned *status, double *freq, void *stream);

/* Kernel launches issued by this solver since creation (own kernels only). */
long long brx_launch_count(const brx_solver *s);

/* Stream the solver launches on (cudaStream_t as void*). */
void *brx_stream(brx_solver *s);

#ifdef __cplusplus
}
#endif
#endif
