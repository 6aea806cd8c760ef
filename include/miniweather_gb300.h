/*
 * miniweather_gb300.h -- C ABI of the GB300 (sm_103a) PyMiniWeather time step.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (cudaStream_t passed as void*, NULL = legacy default stream), launches its
 * kernels on that stream and returns without synchronising.  Nothing here
 * allocates device memory: temporaries are caller-provided workspaces.
 *
 * Layout (the reference's Fields, pyminiweather/data/fields.py:58-123):
 *   state arrays   : (4, nz+4, nx+4) C order, variables DENS=0 UMOM=1 WMOM=2
 *                    RHOT=3 (pyminiweather/__init__.py:14-18), 2-cell halo;
 *   hy_dens_cell, hy_dens_theta_cell             : (nz+4) FP64;
 *   hy_dens_int, hy_dens_theta_int, hy_pressure_int : (nz+1) FP64.
 * Backgrounds stay FP64 for every storage type.
 *
 * Return value: MW_OK (0) or one of the MW_ERR_* codes below; the message of
 * the last failure on the calling thread is given by mw_last_error().
 * Requirements checked before any launch: nx >= 2 (the periodic halo is two
 * cells wide), nz >= 1, 4*(nx+4)*(nz+4) < 2^40, non-NULL pointers, naturally
 * aligned FP64 / FP32 arrays, finite positive dx, dz and time steps.
 */
#ifndef MINIWEATHER_GB300_H
#define MINIWEATHER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MW_ABI_VERSION 4

enum mw_status {
  MW_OK = 0,
  MW_ERR_INVALID_ARG = 1, /* NULL pointer, non-finite or non-positive scalar, bad enum */
  MW_ERR_SHAPE = 2,       /* grid sizes outside the supported range */
  MW_ERR_ALIGN = 3,       /* misaligned pointer */
  MW_ERR_ALIAS = 4,       /* output overlaps an input it must not overlap */
  MW_ERR_CUDA = 5,        /* a CUDA call or kernel launch failed */
  MW_ERR_WORKSPACE = 6,   /* workspace too small */
  MW_ERR_NONFINITE = 7    /* a device-side check found NaN or Inf */
};

enum mw_direction { MW_DIR_X = 0, MW_DIR_Z = 1 }; /* ics/directions.py:4-6 */

/* Arithmetic of the FP64-storage direction-stage kernels. */
enum mw_f64_mode {
  MW_F64_NATIVE = 0, /* IEEE FP64, the reference's formulas as written (a pow
                        and three divides per interface) */
  MW_F64_SPLIT = 1,  /* FP64 loads/stores and update, interior arithmetic in
                        pairs of FP32: about 47 significant bits, FP32 exponent
                        range -- NOT IEEE FP64 arithmetic */
  MW_F64_IEEE = 2    /* IEEE FP64 arithmetic throughout with the fewest FP64
                        operations: 1/rho by a Newton step, the pressure
                        perturbation by its binomial series, values scaled by
                        12 (no divisions per cell) */
};

/* Flags of the direction-stage and step entry points. */
#define MW_FLAG_WRITE_HALO 1u /* write the halo cells into the forcing array
                                 as set_bc_x / set_bc_z do (ics/bcs.py:8-148) */
#define MW_FLAG_INDEX64 2u    /* split form: use the 64-bit-index kernels even
                                 when 32-bit indices suffice (for testing; arrays
                                 of 2^31 or more values always use them) */
#define MW_FLAG_CHECK_FINITE 4u /* mw_step_f64 / _f32 / _f64_host / _f64_noalloc: after the
                                 steps, count the non-finite interior values of
                                 the state and return MW_ERR_NONFINITE if there
                                 are any (synchronises the stream to read the
                                 count, which is kept in the first 8 bytes of
                                 the scratch array: nothing is allocated) */

#define MW_FLAG_PAIRS_OUT 8u /* mw_dirstage_f64, split form: store `out` as the double-FP32
                              pairs mw_step_f64 keeps its first RK stage's result in
                              (needs init == forcing) */
#define MW_FLAG_PAIRS_IN 16u  /* mw_dirstage_f64, split form: read `forcing` as such pairs.
                              With these two flags a caller can issue a split-form step
                              stage by stage with the launches mw_step_f64 makes (to
                              time them one by one); the pair arrays are not FP64 data */

/* Background profile of the initial condition. */
enum mw_background {
  MW_BG_CONST_THETA = 0, /* hydro_const_theta, ics/initial_conditions.py:26-52 */
  MW_BG_BVFREQ = 1       /* hydro_const_bvfreq with N = 0.02, initial_conditions.py:54-81 */
};

#define MW_MAX_BUBBLES 8

const char* mw_last_error(void);
const char* mw_status_string(int status);
int mw_abi_version(void);

/* ---------------------------------------------------------------------------
 * One direction-stage: replaces discrete_step (pyminiweather/solve/step.py:21-82)
 * with set_bc_x/z (ics/bcs.py:8-148), interpolate_x/z, compute_flux_x/z,
 * compute_tend_x/z (solve/interpolate.py:10-250) and add_source_terms
 * (solve/source.py:53-75) fused into one kernel:
 *   out[interior] = init[interior] + dt_stage * tend(forcing)
 * The halo is synthesised from the periodic (x) / wall (z) rule; halo cells
 * of the arrays are never read.  dt_full is params["dt"] (the hyperviscosity
 * time scale, interpolate.py:99-101,147-149).  src_w (nz, nx) is the optional
 * forcing added to the w tendency (the gravity-wave source), NULL for none.
 * `out` may equal `init`; it must not overlap `forcing` (MW_ERR_ALIAS).
 * ------------------------------------------------------------------------- */
int mw_dirstage_f64(int nx, int nz, double dx, double dz, double dt_full, const double* hy_dens_cell,
                    const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                    const double* hy_pressure_int, const double* src_w, const double* init, double* forcing,
                    double* out, double dt_stage, int direction, int f64_mode, unsigned flags, void* stream);

/* FP32 perturbation fields (precision form); backgrounds FP64, converted per row. */
int mw_dirstage_f32(int nx, int nz, double dx, double dz, double dt_full, const double* hy_dens_cell,
                    const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                    const double* hy_pressure_int, const double* src_w, const float* init, float* forcing,
                    float* out, double dt_stage, int direction, unsigned flags, void* stream);

/* ---------------------------------------------------------------------------
 * nsteps full time steps: replaces evolve (pyminiweather/solve/step.py:85-143).
 * Per step the direction order is [Z, X] when *reverse == 0 and [X, Z] when 1
 * (the reference's module-global reverse_direction), toggled after each step;
 * *reverse is a host int updated in place.  Per direction the three RK stages
 * run with dt/3, dt/2, dt:
 *   scratch = S + dt/3 L(S);  state_tmp = S + dt/2 L(scratch);  S = S + dt L(state_tmp)
 * so state_tmp ends holding what the reference's state_tmp holds.  scratch is
 * a third state-sized array (the fused kernel cannot update in place); its
 * contents after the call are unspecified (in the split form each 8-byte slot
 * holds the first stage's result as a pair of floats, not a double).  dt is
 * evolve's time step; dt_full is params["dt"], the hyperviscosity time scale
 * (the reference uses both, step.py:85 and interpolate.py:99-101).
 * ------------------------------------------------------------------------- */
int mw_step_f64(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hy_dens_cell,
                const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                const double* hy_pressure_int, const double* src_w, double* state, double* state_tmp,
                double* scratch, int nsteps, int* reverse, int f64_mode, unsigned flags, void* stream);

/* One time step of a state held in HOST memory (no counterpart in the
 * reference, whose arrays are host arrays to begin with): h_in (4, nz+4, nx+4)
 * is copied into state, the step runs as mw_step_f64 with nsteps = 1, and the
 * resulting state is copied into h_out (which may equal h_in).  Enqueued on
 * `stream`; h_out is complete once the stream is.  In the IEEE-FP64 and split
 * forms the copies overlap the computation by nbands row bands (at most 64 and
 * at most nz / 16); the results are those of copy-in, mw_step_f64, copy-out
 * bit for bit.
 * h_in / h_out should be page-locked for the copies to run asynchronously.
 * Calls on one device share internal copy and compute streams (the x stages
 * of a band run on one beside the caller's) and are serialised. */
int mw_step_f64_host(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hy_dens_cell,
                     const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                     const double* hy_pressure_int, const double* src_w, const double* h_in, double* h_out,
                     double* state, double* state_tmp, double* scratch, int* reverse, int f64_mode, unsigned flags,
                     int nbands, void* stream);

int mw_step_f32(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hy_dens_cell,
                const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                const double* hy_pressure_int, const double* src_w, float* state, float* state_tmp, float* scratch,
                int nsteps, int* reverse, unsigned flags, void* stream);

/* ---------------------------------------------------------------------------
 * mw_step_f64 for callers that cannot allocate device memory.  No counterpart
 * in the reference: it exists for hosts that own every buffer they hand over
 * (a Fortran or C model embedding the solver, a custom call in a framework
 * that pre-allocates all buffers, a real-time loop that forbids allocation
 * once running) and so cannot supply mw_step_f64's third state-sized array.
 * That array is instead a fixed device array inside this library, sized for
 * grids up to 512 x 256 cells ((nx+4)(nz+4) <= 134160); larger grids return
 * MW_ERR_WORKSPACE with the limit in mw_last_error().  Every GPU that loads
 * the library holds the array (4.3 MB) until the process exits.  The first
 * call on each device looks up the array's device address (once per device,
 * with that device current); make that first call before any stream capture.
 * The address is kept for the life of the process, so do not reset a device
 * (cudaDeviceReset) while this entry point is in use on it.
 * All calls share the one array and nothing in it needs to start at zero:
 * calls that overlap on the GPU (other streams, other host threads) race on
 * it, so issue them one after another.  Arguments and results are those of
 * mw_step_f64 without `scratch`, MW_FLAG_CHECK_FINITE included (its counter
 * lives in the same array); it never calls cudaMalloc or cudaFree.
 * ------------------------------------------------------------------------- */
int mw_step_f64_noalloc(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hy_dens_cell,
                        const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                        const double* hy_pressure_int, const double* src_w, double* state, double* state_tmp,
                        int nsteps, int* reverse, int f64_mode, unsigned flags, void* stream);

/* ---------------------------------------------------------------------------
 * Ensembles of uneven grids.  No counterpart in the reference (one grid per
 * process there): many members, each a full simulation with its own nx, nz,
 * dx, dz and dt, advance together, one persistent kernel launch per
 * direction-stage walking a work list over all members.  Each member's state
 * is a (4, nz+4, nx+4) block at state_off (elements) in the shared state,
 * state_tmp and scratch buffers; its backgrounds sit at cell_off (nz+4
 * values) and int_off (nz+1 values) in the shared background buffers.  dt is
 * the member's params["dt"]: the RK step and the hyperviscosity time scale.
 * ------------------------------------------------------------------------- */
typedef struct mw_ens_member {
  int nx, nz;
  double dx, dz, dt;
  long long state_off, cell_off, int_off;
} mw_ens_member;

typedef struct mw_ens_plan_info {
  int n_members, n_x_items, n_z_items, z_tile;
  size_t members_off, x_items_off, z_items_off, bytes; /* byte offsets / size of the device plan */
  size_t xrows_off;    /* split form: per-row background constants, written by each step call */
  long long n_xrows;   /* entries of that table: the length of the cell-centre backgrounds used;
                          the members' stage constants follow it, up to `bytes` */
} mw_ens_plan_info;

/* Size and layout of the work plan for these members (host array) with z
 * work items of z_tile rows (1..64). */
int mw_ensemble_plan_info(int n_members, const mw_ens_member* members, int z_tile, mw_ens_plan_info* info);
/* Write the plan into plan_device (info.bytes bytes, 16-byte aligned); the
 * copy to the device is synchronous.  The plan's work lists are sorted by
 * decreasing cost and handed out by a cursor kept in the plan (the persistent
 * warps and CTAs take the next item as they become free), so a plan serves one
 * step call at a time: calls that use one plan must be ordered (one stream). */
int mw_ensemble_plan(int n_members, const mw_ens_member* members, int z_tile, void* plan_device, size_t plan_bytes,
                     mw_ens_plan_info* info, void* stream);
/* nsteps time steps of every member: 6 persistent launches per step, grid_x
 * and grid_z CTAs (0 = one full-occupancy wave); the FP64 call first writes
 * the plan's row-constant table (one more launch per call).  The direction order follows
 * *reverse as in mw_step_f64 (all members alike).  FP64 storage supports
 * f64_mode MW_F64_IEEE and MW_F64_SPLIT. */
int mw_ensemble_step_f64(void* plan_device, const mw_ens_plan_info* info, const double* hy_dens_cell,
                         const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                         const double* hy_pressure_int, double* state, double* state_tmp, double* scratch, int nsteps,
                         int* reverse, int f64_mode, unsigned flags, int grid_x, int grid_z, void* stream);
/* Resident CTAs per SM of the persistent ensemble kernels of one form (0: FP64
 * storage, split form; 1: FP32 storage; 2: FP64 storage, IEEE-FP64 form) and
 * direction: a default grid is this times the SM count. */
int mw_ensemble_occupancy(int form, int direction, int* blocks_per_sm);
int mw_ensemble_step_f32(void* plan_device, const mw_ens_plan_info* info, const double* hy_dens_cell,
                         const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                         const double* hy_pressure_int, float* state, float* state_tmp, float* scratch, int nsteps,
                         int* reverse, unsigned flags, int grid_x, int grid_z, void* stream);

/* ---------------------------------------------------------------------------
 * Adjoint of one direction-stage (no counterpart in the reference, which has
 * no derivatives): for out = init + dt_stage * L(forcing) as mw_dirstage_f64
 * computes it, given g_out = dJ/d(out) on the interior cells,
 *   g_dst = g_base_a + g_base_b + (add_g_out ? g_out : 0)
 *           + dt_stage * (dL/d forcing)^T g_out
 * on the interior, 0 on the halo.  The transposed map includes the halo rules
 * (a halo value's adjoint returns to the cell it was copied or scaled from),
 * the hyperviscosity and the gravity term.  Arrays are (4, nz+4, nx+4) FP64;
 * a base may be g_dst itself (accumulation); g_dst must not overlap g_out or
 * forcing.  f64_mode: MW_F64_NATIVE (FP64 arithmetic, the reference's
 * formulas: an interface kernel then a gather), MW_F64_IEEE (FP64 arithmetic
 * with the fewest operations, after a small background-table kernel: one
 * kernel in x, an interface kernel then the gather in z) or MW_F64_SPLIT
 * (double-FP32 interior arithmetic as the split forward, one kernel after a
 * small background-table kernel).
 * workspace: mw_dirstage_vjp_workspace_bytes.
 * ------------------------------------------------------------------------- */
size_t mw_dirstage_vjp_workspace_bytes(int nx, int nz);
int mw_dirstage_vjp_f64(int nx, int nz, double dx, double dz, double dt_full, const double* hy_dens_cell,
                        const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                        const double* hy_pressure_int, const double* forcing, const double* g_out,
                        const double* g_base_a, const double* g_base_b, int add_g_out, double* g_dst, double dt_stage,
                        int direction, int f64_mode, void* workspace, size_t workspace_bytes, void* stream);

/* One time step (as mw_step_f64 with nsteps = 1) that also keeps its six
 * stage forcing states in `stages` (6 state arrays, contiguous): for the two
 * directions in order, the direction's input S and its stage states s1, s2.
 * No halo writes.  For the adjoint. */
int mw_step_record_f64(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hy_dens_cell,
                       const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                       const double* hy_pressure_int, const double* src_w, const double* state_in, double* stages,
                       double* state_out, int reverse, int f64_mode, void* stream);
/* Adjoint of one time step recorded by mw_step_record_f64: g_in = dJ/d(state_in)
 * from g_out = dJ/d(state_out) (both (4, nz+4, nx+4), halo 0).  gbuf: 3 state
 * arrays of work space (contiguous); g_in may equal g_out.  f64_mode as for
 * mw_dirstage_vjp_f64. */
int mw_step_vjp_f64(int nx, int nz, double dx, double dz, double dt_full, double dt, const double* hy_dens_cell,
                    const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                    const double* hy_pressure_int, const double* stages, const double* g_out, double* g_in,
                    double* gbuf, int reverse, int f64_mode, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Initial condition: replaces init (pyminiweather/ics/initial.py:11-105):
 * 3x3 Gauss-Legendre cell averages over all (nz+4)(nx+4) cells of the bubbles
 * (sample_ellipse_cosine, utils/utils.py:5-51), plus the hydrostatic
 * backgrounds at cell centres and interfaces, all in FP64.  bubbles is a HOST
 * array of nbubble x (amplitude, x0, z0, xrad, zrad); u0 is the constant
 * initial wind (15 m/s for the gravity-wave case, 0 otherwise).
 * The _f32 form computes in FP64 and rounds the state once at the end.
 * ------------------------------------------------------------------------- */
int mw_init_f64(int nx, int nz, double xlen, double zlen, int background, double u0, int nbubble,
                const double* bubbles, double* state, double* hy_dens_cell, double* hy_dens_theta_cell,
                double* hy_dens_int, double* hy_dens_theta_int, double* hy_pressure_int, void* stream);
int mw_init_f32(int nx, int nz, double xlen, double zlen, int background, double u0, int nbubble,
                const double* bubbles, float* state, double* hy_dens_cell, double* hy_dens_theta_cell,
                double* hy_dens_int, double* hy_dens_theta_int, double* hy_pressure_int, void* stream);

/* GravityBCSourceTerm (pyminiweather/solve/source.py:20-50): src_w (nz, nx) =
 * sample_ellipse_cosine(cell centres, 0.01, xlen/8, 1000, 500, 500) * hy_dens_cell. */
int mw_gravity_source_f64(int nx, int nz, double xlen, double zlen, const double* hy_dens_cell, double* src_w,
                          void* stream);

/* ---------------------------------------------------------------------------
 * Domain totals: replaces compute_stats (pyminiweather/post/stats.py:8-35).
 * out2 (device, 2 doubles) receives (total mass, total energy), summed in FP64
 * in a fixed order (deterministic).  workspace must hold
 * mw_stats_workspace_bytes(nx, nz) bytes.
 * ------------------------------------------------------------------------- */
/* Bounds-checked build (compiled with MW_CHECK=1, python -m pyminiweather_gb300.build
 * --check): every kernel of the library counts each array index outside its
 * array instead of accessing it.  mw_debug_oob_count adds up
 * that count (and resets it if asked); mw_debug_oob_selftest launches one
 * deliberately out-of-range access that the check diverts (the count goes up by
 * one).  Both fail with MW_ERR_INVALID_ARG in the normal build. */
int mw_debug_oob_count(unsigned long long* count, int reset);
int mw_debug_oob_selftest(void* stream);

/* Bounded waits: the kernels that wait on an mbarrier for asynchronous copies
 * (the FP32 x and z passes) give up after a bounded number of rounds instead of
 * hanging, abandon their tile and count it here; *count receives the count
 * (reset to 0 if asked).  Zero unless a copy failed to arrive. */
int mw_debug_wait_timeouts(unsigned long long* count, int reset);

/* FP64 pipe throughput of the current device (no counterpart in the
 * reference; the denominator of the FP64-pipe roofline of the IEEE-FP64
 * form): blocks_per_sm x SMs CTAs of 256 threads, each thread 8 independent
 * FMA chains of iters x 16 steps, timed with CUDA events on `stream`; blocks
 * until done.  *ops_per_second receives FP64 operations per second (an FMA
 * counts as one operation, as in the kernels' operation counts). */
int mw_fp64_throughput(int blocks_per_sm, int iters, double* ops_per_second, void* stream);

/* Count the non-finite (NaN, +-Inf) interior values of a (4, nz+4, nx+4)
 * state into *count (a device counter, added to, not reset); no host sync. */
int mw_count_nonfinite_f64(int nx, int nz, const double* state, unsigned long long* count, void* stream);
int mw_count_nonfinite_f32(int nx, int nz, const float* state, unsigned long long* count, void* stream);

size_t mw_stats_workspace_bytes(int nx, int nz);
int mw_stats_f64(int nx, int nz, double dx, double dz, const double* hy_dens_cell, const double* hy_dens_theta_cell,
                 const double* state, void* workspace, size_t workspace_bytes, double* out2, void* stream);
int mw_stats_f32(int nx, int nz, double dx, double dz, const double* hy_dens_cell, const double* hy_dens_theta_cell,
                 const float* state, void* workspace, size_t workspace_bytes, double* out2, void* stream);

/* compute_solution_variables (pyminiweather/post/stats.py:38-69): out (4, nz, nx)
 * = (rho', u, w, theta'). */
int mw_solution_variables_f64(int nx, int nz, const double* hy_dens_cell, const double* hy_dens_theta_cell,
                              const double* state, double* out, void* stream);

/* Text dump of the reference's driver (pyminiweather/__main__.py:220-233,
 * np.savetxt(outfile, array.reshape(-1, last_dim), delimiter=",")): rows x cols
 * HOST values, each "%.18e" as np.savetxt writes it ("nan", "inf", "-inf" for
 * the special values), "," between values, "\n" after each row; the file is
 * created (append = 0) or appended to.  threads <= 0: all hardware threads.
 * Byte-identical to np.savetxt's output. */
int mw_savetxt_f64(const double* values, long long rows, long long cols, const char* path, int append, int threads);

/* ---------------------------------------------------------------------------
 * Unfused pieces of one direction-stage, for callers that use the reference's
 * fine-grained functions.  Intermediate shapes follow data/fields.py:67-78.
 * ------------------------------------------------------------------------- */
/* set_bc_x / set_bc_z (ics/bcs.py:8-39, 67-148), in place on `state`. */
int mw_set_bc_f64(int nx, int nz, const double* hy_dens_cell, double* state, int direction, void* stream);
/* interpolate_x (vals, d3: (4, nz, nx+1)) / interpolate_z ((4, nz+1, nx)),
 * solve/interpolate.py:10-79; reads the halo cells of `state` as stored. */
int mw_interpolate_f64(int nx, int nz, const double* state, double* vals, double* d3, int direction, void* stream);
/* compute_flux_x / compute_flux_z (solve/interpolate.py:82-186): flux (4, nz+1, nx+1);
 * the z form zeroes d3[DENS] at interfaces 0 and nz in place, as the reference does. */
int mw_flux_f64(int nx, int nz, double dx, double dz, double dt_full, const double* hy_dens_cell,
                const double* hy_dens_theta_cell, const double* hy_dens_int, const double* hy_dens_theta_int,
                const double* hy_pressure_int, const double* vals, double* d3, double* flux, int direction,
                void* stream);
/* compute_tend_x / compute_tend_z (solve/interpolate.py:189-250) plus the
 * optional src_w forcing: tend (4, nz, nx). */
int mw_tend_f64(int nx, int nz, double dx, double dz, const double* flux, const double* state_forcing,
                const double* src_w, double* tend, int direction, void* stream);
/* add_source_terms (pyminiweather/solve/source.py:53-75) for the gravity-wave
 * case: tend[WMOM] += src_w. */
int mw_add_source_f64(int nx, int nz, const double* src_w, double* tend, void* stream);
/* The stage update of discrete_step (solve/step.py:80-82). */
int mw_update_f64(int nx, int nz, const double* init, const double* tend, double* out, double dt_stage, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MINIWEATHER_GB300_H */
