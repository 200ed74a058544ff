/*
 * flow_gb300.h -- C ABI of the GB300 (sm_103a) kernel set for the flow
 * mini-app.
 *
 * Part 1 is the reference's own kernel-set interface, with identical names,
 * argument order and meaning, so that an unmodified host driver (main.c) can
 * select this set the way it selects omp3 or cuda (`KERNELS=gb300`).  Part 2
 * adds status-returning control functions.  Part 3 is the mixed-precision
 * form.
 *
 * Memory: every array argument is a DEVICE pointer (as for the reference cuda
 * set).  The Mesh struct is host memory; its edgedx/edgedy/celldx/celldy
 * arrays are device pointers; mesh->dt and mesh->dt_h are host doubles that
 * set_timestep and solve_hydro_2d update before returning.  The kernel set
 * never allocates: its only device scratch is the caller's reduce_array,
 * which must hold at least local_nx*local_ny doubles (the arch default).
 *
 * Errors: the reference entry points return void and abort on a CUDA error
 * (cuda/flow.cu:24 gpu_check).  Here they record the error instead; read it
 * with gb300_last_error()/gb300_last_error_message().  A failed call leaves
 * the mesh scalars unchanged.
 *
 * Scope: one rank (all Mesh::neighbours must be FLOW_EDGE); pad >= 2 and at
 * least 2 interior cells per axis.
 */
#ifndef FLOW_GB300_H
#define FLOW_GB300_H

#include "flow_mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ===== Part 1: the reference kernel-set interface ======================== */

/* One timestep (replaces flow_interface.h:16-20; omp3/flow.c:10-52). */
void solve_hydro_2d(Mesh* mesh, int tt, double* P, double* rho,
                    double* rho_old, double* e, double* u, double* v,
                    double* rho_u, double* rho_v, double* Qxx, double* Qyy,
                    double* F_x, double* F_y, double* uF_x, double* uF_y,
                    double* vF_x, double* vF_y, double* reduce_array);

/* CFL timestep and leapfrog dt/dt_h update (flow_interface.h:23-26;
 * omp3/flow.c:73-106).  Blocks until mesh->dt/dt_h are updated. */
void set_timestep(const int nx, const int ny, double* Qxx, double* Qyy,
                  const double* rho, const double* e, Mesh* mesh,
                  double* reduce_array, const int first_step,
                  const double* celldx, const double* celldy);

/* Interior totals of rho and rho*e, printed on rank 0 when verbose
 * (flow_interface.h:29-30; omp3/flow.c:973-995). */
void print_conservation(const int nx, const int ny, double* rho, double* e,
                        double* reduce_array, Mesh* mesh);

/* Stage entry points (omp3/flow.h:4-88), each with its ghost fills. */
void equation_of_state(const int nx, const int ny, double* P, const double* rho,
                       const double* e); /* omp3/flow.h:4 */
void pressure_acceleration(const int nx, const int ny, Mesh* mesh,
                           const double dt, double* rho_u, double* rho_v,
                           double* u, double* v, const double* P,
                           const double* rho, const double* edgedx,
                           const double* edgedy, const double* celldx,
                           const double* celldy); /* omp3/flow.h:9 */
void artificial_viscosity(const int nx, const int ny, Mesh* mesh,
                          const double dt, double* Qxx, double* Qyy, double* u,
                          double* v, double* rho_u, double* rho_v,
                          const double* rho, const double* edgedx,
                          const double* edgedy, const double* celldx,
                          const double* celldy); /* omp3/flow.h:16 */
void shock_heating_and_work(const int nx, const int ny, Mesh* mesh,
                            const double dt_h, double* e, const double* P,
                            const double* u, const double* v, const double* rho,
                            const double* Qxx, const double* Qyy,
                            const double* celldx,
                            const double* celldy); /* omp3/flow.h:24 */
void advect_mass_and_energy(const int nx, const int ny, Mesh* mesh,
                            const int tt, const double dt, const double dt_h,
                            double* rho, double* e, double* rho_old,
                            double* F_x, double* F_y, double* eF_x,
                            double* eF_y, const double* u, const double* v,
                            const double* edgedx, const double* edgedy,
                            const double* celldx,
                            const double* celldy); /* omp3/flow.h:31 */
void momentum_x_flux_in_x(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* velocity_x, double* uF_x,
                          const double* mass_flux_x, const double* edgedx,
                          const double* edgedy,
                          const double* celldx); /* omp3/flow.h:40 */
void momentum_x_flux_in_y(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* velocity_x,
                          double* velocity_y, double* uF_y,
                          const double* mass_flux_y, const double* edgedx,
                          const double* edgedy,
                          const double* celldy); /* omp3/flow.h:46 */
void momentum_y_flux_in_x(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, const double* velocity_x,
                          double* velocity_y, double* vF_x,
                          const double* mass_flux_x, const double* edgedx,
                          const double* celldy,
                          const double* celldx); /* omp3/flow.h:53 */
void momentum_y_flux_in_y(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* velocity_y, double* vF_y,
                          const double* mass_flux_y, const double* edgedy,
                          const double* celldx,
                          const double* celldy); /* omp3/flow.h:60 */
void advect_momentum(const int nx, const int ny, const int tt, Mesh* mesh,
                     const double dt_h, const double dt, double* u, double* v,
                     double* uF_x, double* uF_y, double* vF_x, double* vF_y,
                     double* rho_u, double* rho_v, const double* rho,
                     const double* F_x, const double* F_y,
                     const double* edgedx, const double* edgedy,
                     const double* celldx,
                     const double* celldy); /* omp3/flow.h:66 */
void x_mass_and_energy_flux(const int nx, const int ny, const int first,
                            Mesh* mesh, const double dt, const double dt_h,
                            double* rho, double* rho_old, double* e,
                            const double* u, double* F_x, double* eF_x,
                            const double* celldx, const double* edgedx,
                            const double* celldy,
                            const double* edgedy); /* omp3/flow.h:75 */
void y_mass_and_energy_flux(const int nx, const int ny, const int first,
                            Mesh* mesh, const double dt, const double dt_h,
                            double* rho, double* rho_old, double* e,
                            const double* v, double* F_y, double* eF_y,
                            const double* celldx, const double* edgedx,
                            const double* celldy,
                            const double* edgedy); /* omp3/flow.h:83 */

/* Reflective ghost fill of one nx x ny device array (the single-rank part of
 * the arch handle_boundary_2d the reference calls 19 times per step, e.g.
 * omp3/flow.c:156).  invert: 0 none, 1 negate across x walls, 2 across y. */
void handle_boundary_2d(const int nx, const int ny, Mesh* mesh, double* arr,
                        const int invert, const int pack);

/* ===== Part 2: control and status ======================================== */

enum {
  GB300_OK = 0,
  GB300_ERR_CUDA = 1,    /* a CUDA call or launch failed */
  GB300_ERR_ARG = 2,     /* unsupported sizes, null pointers, multi-rank */
  GB300_ERR_TIMEOUT = 3, /* a bounded device wait ran out */
  GB300_ERR_STATE = 4    /* device-side status word reported a fault */
};

/* Timestep implementations selectable for solve_hydro_2d. */
enum {
  GB300_MODE_EXACT = 0,      /* the stage entry points in sequence; bit-exact
                                with the reference omp3 set */
  GB300_MODE_FUSED = 1,      /* fused kernels, FP64, within 1e-12 of the
                                reference; the default */
  GB300_MODE_FUSED_LAG = 2   /* the same step with the Lagrangian phase
                                (omp3/flow.c:22-38) as one kernel (TMA-staged,
                                ~43 B/cell of DRAM traffic instead of ~165);
                                the same numbers bit for bit */
};

int gb300_last_error(void);
const char* gb300_last_error_message(void);
void gb300_clear_error(void);

/* Stream every launch of this thread goes to (default: the legacy stream). */
int gb300_set_stream(void* stream);
void* gb300_get_stream(void);

int gb300_set_mode(int mode);
int gb300_get_mode(void);

/* Output rows per CTA of the one-kernel Lagrangian phase of
 * GB300_MODE_FUSED_LAG (1 .. 64, default 32): a tuning knob; every value gives
 * the same numbers.  No reference counterpart (the reference has no tiles). */
int gb300_set_lagrangian_rows(int rows);

/* Domain decomposition (the arch layer's MPI DECOMP, Makefile:47-59: each
 * rank a band of the mesh, halo layers exchanged in every
 * handle_boundary_2d(..., PACK), e.g. omp3/flow.c:156-157, and the dt
 * minimum reduced by reduce_all_min, omp3/flow.c:100).  A rank whose Mesh
 * has a neighbour that is a rank (neighbours[k] != FLOW_EDGE) runs in
 * GB300_MODE_EXACT, with its ghost layers filled as the single-rank step
 * fills them: physical x walls over the interior rows, then the exchange,
 * then physical y walls over whole rows.  The caller supplies the transport:
 *   halo(ctx, mesh, arr, w, h, invert) fills the ghost layers of the w x h
 *     device array arr that face neighbouring ranks (pad rows/columns, full
 *     width) from those ranks' interior values, synchronously; the library
 *     has synchronised its stream before the call.  Returns 0 on success.
 *   reduce_min(ctx, &value) replaces value by its minimum over the ranks.
 * flow_gb300/decomp.py gives both over torch.distributed and over threads
 * sharing one GPU.  Results match the single-rank exact step bit for bit. */
typedef int (*gb300_halo_fn)(void* ctx, const Mesh* mesh, double* arr, int w, int h,
                             int invert);
typedef int (*gb300_reduce_min_fn)(void* ctx, double* value);
int gb300_set_halo_exchange(gb300_halo_fn fn, void* ctx);
int gb300_set_reduce_min(gb300_reduce_min_fn fn, void* ctx);

/* Kernel launches this library has issued for the fused timestep and the
 * conservation totals since it was loaded (a counter a benchmark reads around
 * its timed region).  No reference counterpart. */
unsigned long long gb300_launch_count(void);

/* 1 (default): print dt and conservation totals as the reference does
 * (omp3/flow.c:18-20, 991-994); 0: silent. */
int gb300_set_verbose(int verbose);

int gb300_synchronize(void);

/* The fused step (both forms) carries from one timestep to the next which
 * tiles of the mesh were at rest, and does not recompute them while they stay
 * so.  It trusts that record only for the step that directly follows (tt one
 * more, the same arrays and reduce_array, no other call of this library that
 * takes a mesh in between).  A caller that writes the state arrays by other
 * means (its own copies or kernels) between two such steps calls this first.
 * No reference counterpart (the reference recomputes every cell). */
int gb300_state_changed(void);

/* Status-returning forms of the Part 1 calls. */
int gb300_solve_hydro_2d(Mesh* mesh, int tt, double* P, double* rho,
                         double* rho_old, double* e, double* u, double* v,
                         double* rho_u, double* rho_v, double* Qxx,
                         double* Qyy, double* F_x, double* F_y, double* uF_x,
                         double* uF_y, double* vF_x, double* vF_y,
                         double* reduce_array);

/* Interior totals: out[0] = sum rho, out[1] = sum rho*e (host array).  With
 * sync = 0 the totals stay in reduce_array[3..4] and out is not written.
 * Where reduce_array holds the fused step's flag region the sums are formed by
 * 128x128 tiles whose partial sums stay there; a call directly after a fused
 * step keeps the partials of the tiles that step left at rest (see
 * gb300_state_changed).  The totals depend only on the cells. */
int gb300_conservation(int nx, int ny, int pad, const double* rho,
                       const double* e, double* reduce_array, double* out,
                       int sync);

/* No counterpart in the reference.  The same interior totals as
 * gb300_conservation (out[0] = sum rho, out[1] = sum rho*e, host array,
 * synchronous on the stream set with gb300_set_stream), for callers that hold only the density
 * and energy arrays and must not allocate device memory: a monitoring or
 * validation hook between timesteps (cudaMalloc/cudaFree would synchronise
 * the whole device and stall other streams' work), or a run whose ensemble
 * fills HBM.  It allocates nothing: its scratch is a fixed 256 KiB
 * __device__ array inside libflow_gb300.so, holding one pair of partial sums
 * per interior row, so meshes with more than GB300_NOALLOC_MAX_ROWS interior
 * rows are rejected with GB300_ERR_ARG.
 *   - Every call looks up the scratch address of the current device with
 *     cudaGetSymbolAddress, so it stays right across a device reset.
 *   - Never call it while its stream is capturing a CUDA graph: it copies the
 *     totals to host memory and synchronises the stream, neither of which a
 *     capture allows.
 *   - The scratch's ticket counter must be zero when the kernel starts: it is
 *     zero at load, every call clears it on the stream before launching, and
 *     the kernel leaves it at zero.
 *   - All calls on one device share the scratch: two calls in flight at once
 *     (different streams or host threads) race and return wrong totals.
 *     Serialise them, or use gb300_conservation with separate reduce_arrays.
 * The additions run in a fixed order (row sums, then rows in order), so the
 * totals can differ from gb300_conservation's in the last bits, and repeated
 * calls on the same state return identical totals. */
#define GB300_NOALLOC_MAX_ROWS 16384
int gb300_conservation_noalloc(int nx, int ny, int pad, const double* rho,
                               const double* e, double* out);

/* Device-side problem set-up (the arch layer's initialise_shared_data_2d
 * step, main.c:52-54): nboxes problem boxes from the params file (host array
 * of nboxes x 6: density, energy, xpos, ypos, width, height; at most
 * GB300_MAX_BOXES) rasterised onto every cell of an nx x ny mesh whose face
 * positions are the device arrays edgex (nx+1) and edgey (ny+1).  A cell
 * takes the last box whose [pos, pos + extent) holds its left / bottom edge
 * coordinate, 0 where none does.  Ghost cells follow the same rule; the
 * caller applies the reflective fill afterwards, as main.c:56-59 does.
 * Asynchronous on the current stream. */
#define GB300_MAX_BOXES 32
int gb300_fill_boxes(int nx, int ny, const double* edgex, const double* edgey,
                     const double* boxes, int nboxes, double* rho, double* e);

/* Per-kernel CUDA-event timing of the fused timestep: enable, run steps,
 * then read one (name, launches, total milliseconds) entry per kernel. */
int gb300_profile_enable(int on);
int gb300_profile_reset(void);
int gb300_profile_count(void);
int gb300_profile_entry(int i, char* name, int name_len, long long* launches,
                        double* total_ms);

/* ===== Part 3: the mixed-precision form ================================== */

/* Same scheme and step sequence as solve_hydro_2d, with FP32 arithmetic for
 * the equation of state, accelerations, viscosity, shock heating, the CFL
 * candidates and all fluxes, and FP64 for the stored density and specific
 * energy, their conservative update in advection, the energy increment of
 * shock heating, the dt minimum and the conservation totals.  Momenta are
 * FP32 face arrays ((nx+1)*(ny+1) floats, same layout as the FP64 ones).
 * Every other array lives in a caller-provided device workspace of
 * gb300_mixed_workspace_bytes() bytes (the form never allocates). */
size_t gb300_mixed_workspace_bytes(int local_nx, int local_ny);

/* Byte offset inside the workspace of the form's FP32 velocities, laid out
 * like the FP64 ones (x faces (nx+1) per row, y faces nx per row):
 * field 0 = u, 1 = v; (size_t)-1 for any other field. */
#define GB300_MIXED_U 0
#define GB300_MIXED_V 1
size_t gb300_mixed_workspace_offset(int local_nx, int local_ny, int field);

/* Zeroes the workspace and derives its FP32 copies of rho and e (whose
 * ghosts must already be filled); with initial_timestep = 1 also performs the
 * driver's first set_timestep (first_step = 0, zero viscous stresses). */
int gb300_mixed_prepare(Mesh* mesh, double* rho, double* e, void* workspace,
                        size_t bytes, double* reduce_array,
                        int initial_timestep);

/* One timestep; updates mesh->dt and mesh->dt_h like solve_hydro_2d. */
int gb300_mixed_solve(Mesh* mesh, int tt, double* rho, double* e, float* rho_u,
                      float* rho_v, void* workspace, size_t bytes,
                      double* reduce_array);

/* ===== Part 4: batched ensembles ========================================== */

/* Many independent problems of different sizes, each with its own dt,
 * advanced together: one persistent cooperative kernel launch per timestep
 * runs every phase of the step over a flattened list of (instance, tile) work
 * items, separated by bounded grid barriers; pairs of steps replay a captured
 * CUDA graph.  precision 0 = FP64 form, 1 = mixed form.  Every instance is a
 * uniform mesh of global_nx x global_ny interior cells (pad 2) over
 * width x height, with reflective walls.  All device memory is one
 * caller-provided pool of gb300_batch_pool_bytes() bytes. */
typedef struct GB300Batch GB300Batch;

int gb300_batch_create(int n, const int* global_nx, const int* global_ny,
                       const double* width, const double* height, int precision,
                       GB300Batch** out);
size_t gb300_batch_pool_bytes(const GB300Batch* batch);
/* Lays the instances out in the pool (zeroed) and builds the work lists. */
int gb300_batch_bind(GB300Batch* batch, void* pool, size_t bytes);
/* Host interior density / specific energy (global_ny x global_nx, row-major)
 * of instance i, ghost fill, and the driver's first set_timestep with the
 * params dt dt_param (main.c:30, 64-66). */
int gb300_batch_set_state(GB300Batch* batch, int i, const double* rho,
                          const double* e, double dt_param);
/* The same from problem boxes rasterised on the device (gb300_fill_boxes
 * rule, on the instance's uniform mesh over width x height): no host arrays
 * and no copies. */
int gb300_batch_fill_boxes(GB300Batch* batch, int i, const double* boxes, int nboxes,
                           double dt_param);
/* Tile height (1..32 rows), CTAs per SM of the persistent launch (0 = as many
 * as fit) and work order (0 largest instance first, 1 input order). */
int gb300_batch_set_tuning(GB300Batch* batch, int rows, int ctas_per_sm,
                           int order);
int gb300_batch_get_tuning(const GB300Batch* batch, int* rows,
                           int* ctas_per_sm, int* order, int* grid);
/* Advances every instance by `steps` timesteps (asynchronous on the current
 * stream); use_graph replays pairs of steps from a captured CUDA graph. */
int gb300_batch_step(GB300Batch* batch, int steps, int use_graph);
/* Synchronises and returns GB300_ERR_TIMEOUT if a grid barrier ran out. */
int gb300_batch_status(GB300Batch* batch);
/* Bound of each grid-barrier wait of the batched kernel, in 64 ns naps
 * (default 2^25, about 2 s): past it the kernel records GB300_ERR_TIMEOUT and
 * every block returns.  No reference counterpart (the reference aborts on a
 * CUDA error, cuda/flow.cu:24). */
int gb300_batch_set_spin_limit(GB300Batch* batch, long long spins);
/* How a batched step is launched.  GB300_BATCH_PHASES (the default): one
 * launch per phase of the step (pressure, viscosity, viscous acceleration,
 * shock heating + CFL, the two sweeps, the four momentum pairs) over the tiles
 * of every instance, plus the per-instance dt rule; each phase kernel has the
 * register budget and copy rings of the single-problem kernel of that phase.
 * GB300_BATCH_PERSISTENT: one cooperative launch per step running every phase
 * with grid barriers between them.  Both give the single-problem numbers bit
 * for bit; both are captured two steps at a time as a CUDA graph.  No
 * reference counterpart. */
enum { GB300_BATCH_PHASES = 0, GB300_BATCH_PERSISTENT = 1 };
int gb300_batch_set_schedule(GB300Batch* batch, int schedule);
int gb300_batch_get_schedule(const GB300Batch* batch);
/* Interior fields (host, optional), dt/dt_h pair and interior totals of rho
 * and rho*e of instance i. */
int gb300_batch_get_state(GB300Batch* batch, int i, double* rho, double* e,
                          double* dt_pair, double* totals);
long long gb300_batch_cells(const GB300Batch* batch);
void gb300_batch_destroy(GB300Batch* batch);

/* Measured FP64 FMA issue rate of the current GPU (FMA instructions per
 * second per GPU), the compute roofline of the FP64 timestep.  Allocates a
 * small scratch buffer; not for use inside stream capture. */
int gb300_measure_fp64_fma_rate(double* fma_per_s);

/* Self-check of the FP64 helpers the fused kernels use in place of IEEE
 * operations, on n hashed inputs (synchronous; allocates a small buffer):
 *   counts[0]  x*0.5 on the integer pipes != IEEE x*0.5 (every bit pattern)
 *   counts[1]  x*2 on the integer pipes != IEEE x*2
 *   counts[2]  power-of-two test wrong
 *   counts[3]  one-Newton-step quotient with one correction != IEEE n/d
 *   counts[4]  one-Newton-step reciprocal, then a corrected quotient != IEEE n/d
 *   counts[5]  x times a power of two on the integer pipes != IEEE product
 *   counts[6]  1/p, x/(2p), 1/(p*p) of powers of two x, p from their
 *              exponent fields != the IEEE expressions
 * max_ulp[0..1]: the largest gaps of counts[3..4] in units in the last
 * place; max_seed_rel_err: the largest |rcp.approx(d) * d - 1|. */
int gb300_check_fp64_helpers(long long n, unsigned long long seed, long long* counts,
                             long long* max_ulp, double* max_seed_rel_err);

#ifdef __cplusplus
}
#endif

#endif /* FLOW_GB300_H */
