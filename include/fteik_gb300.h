/*
 * fteik_gb300 C ABI: the drop-in boundary of fteikpy's traveltime path.
 *
 * Every entry point takes plain pointers and sizes. Arrays named "device" live
 * in GPU memory owned by the caller; the library never allocates memory for
 * results or scratch (the caller passes a workspace of the size the matching
 * *_workspace_bytes function returns). `stream` is a cudaStream_t (NULL = the
 * legacy default stream). Arrays use the reference's C-order layouts:
 * cells [nz][nx](ny), nodes [nz+1][nx+1](ny+1), gradients [nodes][ndim],
 * batched arrays with a leading source axis.
 *
 * Return value: 0 on success, else one of FTEIK_* below. The blocking calls
 * synchronise `stream` before returning so that device-side failures (a ray
 * hitting max_step, a dependency wait that timed out) are reported.
 */
#ifndef FTEIK_GB300_H
#define FTEIK_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FTEIK_OK 0
#define FTEIK_SOURCE_OUT_OF_BOUND 1   /* ValueError("source out of bound") */
#define FTEIK_END_POINT_OUT_OF_BOUND 2 /* ValueError("end point out of bound") */
#define FTEIK_MAX_STEP_REACHED 3      /* RuntimeError("maximum number of steps reached") */
#define FTEIK_DEVICE_WAIT_TIMEOUT 4   /* a bounded device-side wait gave up */
#define FTEIK_INVALID_ARGUMENT 5
#define FTEIK_CUDA_ERROR 6
#define FTEIK_WORKSPACE_TOO_SMALL 7
#define FTEIK_TAPE_OVERFLOW 8         /* the adjoint's tape needs more history slots */

/* Library version and a short description of the last CUDA error, if any. */
const char* fteik_version(void);
const char* fteik_last_error(void);

/* Measurement hooks (no counterpart in the reference, which has no timing).
 * fteik_kernel_timing(1) makes the 3D solve record CUDA events around its
 * sweep kernel on the launching stream; fteik_last_sweep_ms then returns that
 * kernel's duration. fteik_fp64_peak times a DFMA loop (nblocks x 256 threads,
 * 4 chains each; `scratch` holds nblocks*256 doubles) and returns FLOP/s. */
int fteik_kernel_timing(int on);
/* Tuning knobs (no counterpart in the reference); -1 chooses automatically.
 * "sweep_coef": 0 makes the 3D sweep derive its slowness factors from the
 * 8 cells around each node, 1 makes it read precomputed coefficient arrays
 * (faster for batches of sources, which reuse them). "sweep_pencil": pencil
 * width along x, 2, 4 or 8. "sweep_chunk": steps between progress
 * publications, a power of 2 up to 64. "sweep_team": 1 runs single-model
 * solves with the team kernel (compacted operators; the default from 4
 * sources), 0 with one warp per pencil. "sweep_keep_test": 0 turns off the
 * test that skips the 2D/3D operators of nodes that provably keep their value
 * (grids with equal spacings only). "adjoint_chunk": steps between progress
 * publications of the adjoint's reverse pass, a power of 2 up to 64.
 * "sweep2d_keys": 0 makes the 2D sweeps compare with IEEE comparisons
 * throughout (by default they use integer order keys for every source whose
 * first propagation left only finite values, where the two agree).
 * "sweep2d_warp": 1 runs each 2D source on a warp (the warp precomputes the
 * terms of each column that do not depend on the previous node, one lane
 * runs the chain; the default up to 4 sources per SM), 0 on one thread, 2
 * on a block of 4 warps (one lane runs the chain while three warps
 * precompute the pass's rows ahead of it; the default up to one source per
 * SM).
 * "sweep2d_speculate": 0 turns off the warp kernel's speculated updates (each
 * row also evaluated with the previous node's value from before the pass,
 * taken when the chain's actual value has the same bits).
 * "ray_lanes": lanes per ray of fteik_ray3d / fteik_ray2d: 32 (a warp per
 * ray; the default up to one ray per SM sub-partition), 4 (the default up to
 * 16384 rays) or 1 (larger launches); honor_grid rays run on 4 or 1.
 * "sweep2d_wait_ns": the bound, in ns, of each wait between the warps of the
 * block-per-source 2D kernel (default 10 s); a wait that reaches it stops
 * the block and the solve returns FTEIK_DEVICE_WAIT_TIMEOUT.
 * Results are identical for every setting.
 * fteik_get_option reads a knob back. */
int fteik_set_option(const char* name, long long value);
int fteik_get_option(const char* name, long long* value);
int fteik_last_sweep_ms(float* ms);
int fteik_fp64_peak(double* scratch, int nblocks, int iters, double* flops_per_s, void* stream);
/* Diagnostic (no counterpart in the reference): out[i] = the square root the
 * kernels use (sqrt_rn, correctly rounded like IEEE sqrt with most of its
 * work off the FP64 pipe) of the n device doubles x[i], on `stream`. */
int fteik_sqrt_rn(const double* x, long long n, double* out, void* stream);
/* Diagnostic (no counterpart in the reference): out[i] = x[i] / c as the
 * kernels divide by a positive constant (div_tk: a product with RN(1/c) and
 * Tuckerman's rounding test, correctly rounded like IEEE division), for the n
 * device doubles x[i], on `stream`.  c must be positive and finite. */
int fteik_div_rn(const double* x, long long n, double c, double* out, void* stream);
/* Diagnostic (no counterpart in the reference): out[i] = 1 / x[i] as the
 * gradient post-pass takes the reciprocal of a gradient's norm (recip_rn,
 * correctly rounded like IEEE division), for the n device doubles x[i]. */
int fteik_recip_rn(const double* x, long long n, double* out, void* stream);

/* ---------------------------------------------------------- model set-up --
 * slowness = 1.0 / velocity, as Eikonal2D/3D.solve does before calling the
 * solver (fteikpy/_solver.py:49-50,120-121), for n values on the device.
 * `flag` is a device int used as scratch. Blocking; returns
 * FTEIK_INVALID_ARGUMENT when a slowness is not finite or lies outside
 * (1e-150, 1e150) (the solver kernels need its square to be a normal double). */
int fteik_slowness(const double* velocity, long long n, double* slow, int* flag, void* stream);

/* ---------------------------------------------------------------- 3D solve --
 * Replaces solve3d / fteik3d / fteik3d_vectorized
 * (fteikpy/_fteik/_fteik3d.py:394-525) as called by Eikonal3D.solve
 * (fteikpy/_solver.py:120-126).
 *
 *  slow      device [nz][nx][ny] slowness (1 / velocity), cell counts nz, nx, ny
 *  sources   HOST   [nsrc][3] source (z, x, y) relative to the grid origin
 *  tt        device [nsrc][nz+1][nx+1][ny+1] traveltimes (output)
 *  grad      0: traveltimes only; 1: also the unit gradients; 2: traveltimes
 *            and the branch record kept in the workspace (no gradients)
 *  ttgrad    device [nsrc][nz+1][nx+1][ny+1][3] unit gradients (output; may be
 *            NULL unless grad == 1)
 *  vzero     device [nsrc] slowness at each source cell (output)
 *  workspace device scratch of at least fteik3d_workspace_bytes(...) bytes
 *  spin_limit maximum polls of one dependency wait before the kernel gives up
 *            with FTEIK_DEVICE_WAIT_TIMEOUT (<= 0: default)
 * All sources are solved by one persistent kernel launch that runs every
 * directional sweep of every source.
 */
size_t fteik3d_workspace_bytes(int nz, int nx, int ny, int nsrc, int grad);
int fteik3d_solve(const double* slow, int nz, int nx, int ny, double dz, double dx, double dy,
                  const double* sources, int nsrc, int nsweep, int grad, double* tt,
                  double* ttgrad, double* vzero, void* workspace, size_t workspace_bytes,
                  long long spin_limit, void* stream);
/* Same work, enqueued on `stream` without waiting; the status is read later
 * with fteik_workspace_status(). Host-side argument errors return at once.
 * Everything it enqueues can be captured in a CUDA graph when `sources` is
 * pinned host memory: a replay copies the sources from that buffer again (so
 * new positions can be written between replays; the bounds check runs at
 * capture time only, so they must stay inside the model) and re-runs every
 * kernel. With kernel timing on, the timing events are captured too. */
int fteik3d_solve_async(const double* slow, int nz, int nx, int ny, double dz, double dx,
                        double dy, const double* sources, int nsrc, int nsweep, int grad,
                        double* tt, double* ttgrad, double* vzero, void* workspace,
                        size_t workspace_bytes, long long spin_limit, void* stream);
/* Synchronise `stream` and return the device-side status of the last solve
 * enqueued with this workspace. */
int fteik_workspace_status(const void* workspace, void* stream);

/* ------------------------------------------------------ batch of 3D models --
 * No single counterpart in the reference: there, each model is an Eikonal3D
 * and each solve a fteik3d_vectorized call (fteikpy/_fteik/_fteik3d.py:493-513)
 * over that model's sources. Here models of different sizes and spacings,
 * each with its own sources, are solved by ONE persistent sweep launch.
 *  slow      HOST [nmodel] array of device pointers, model m [nz][nx][ny]
 *  dims      HOST [nmodel][3] cell counts (nz, nx, ny), each >= 2
 *  spacing   HOST [nmodel][3] (dz, dx, dy)
 *  sources   HOST [sum nsrc][3], model by model, relative to each origin
 *  nsrc      HOST [nmodel] sources per model (>= 1)
 *  tt        HOST [nmodel] array of device pointers, model m
 *            [nsrc[m]][nz+1][nx+1][ny+1]
 *  ttgrad    HOST [nmodel] array of device pointers ([..][3]) or NULL when
 *            grad == 0 (grad is 0 or 1 here)
 *  vzero     device [sum nsrc]
 *  workspace device scratch of fteik3d_batch_workspace_bytes(...) bytes
 * Results equal those of one fteik3d_solve per model. Blocking. */
size_t fteik3d_batch_workspace_bytes(int nmodel, const int* dims, const int* nsrc, int grad);
int fteik3d_solve_batch(int nmodel, const double* const* slow, const int* dims,
                        const double* spacing, const double* sources, const int* nsrc,
                        int nsweep, int grad, double* const* tt, double* const* ttgrad,
                        double* vzero, void* workspace, size_t workspace_bytes,
                        long long spin_limit, void* stream);

/* ----------------------------------------------------------------- autotuner --
 * Launch shape of the 3D sweep kernel: pencil width along x (2, 4 or 8; a
 * pencil is w x 32/w node columns, one per lane of a warp), steps between
 * progress publications (a power of 2, the hyperplane chunk), and the
 * coefficient source (1 precomputed arrays, 0 slowness cells), and team mode
 * (1: blocks of 4 sources step through a pencil together and evaluate the
 * 2D/3D operators their lanes need packed 32 to a warp instruction; single
 * model only). The autotuner
 * times candidate shapes on the caller's problem (one sweep per direction,
 * sweep kernel only), keeps the fastest for that problem signature (cell
 * counts, source counts, gradients) for the rest of the process, and returns
 * it in shape[4] = {pencil, chunk, coef, team} and its time in best_ms.
 * Solves of the same signature then use it unless fteik_set_option overrides
 * a part ("sweep_pencil", "sweep_chunk", "sweep_coef", "sweep_team";
 * -1 = automatic). The
 * arguments are those of fteik3d_solve / fteik3d_solve_batch (the outputs are
 * overwritten). No counterpart in the reference. */
int fteik3d_autotune(const double* slow, int nz, int nx, int ny, double dz, double dx, double dy,
                     const double* sources, int nsrc, int grad, double* tt, double* ttgrad,
                     double* vzero, void* workspace, size_t workspace_bytes, long long spin_limit,
                     int* shape, float* best_ms, void* stream);
int fteik3d_batch_autotune(int nmodel, const double* const* slow, const int* dims,
                           const double* spacing, const double* sources, const int* nsrc,
                           int grad, double* const* tt, double* const* ttgrad, double* vzero,
                           void* workspace, size_t workspace_bytes, long long spin_limit,
                           int* shape, float* best_ms, void* stream);
/* Forget every measured shape. */
int fteik_clear_tuning(void);
/* Name of the sweep kernel the last 3D solve on this host thread launched
 * ("sweep3d_team_kernel", "sweep3d_kernel", "sweep3d_kernel (models)"). */
const char* fteik_last_sweep_kernel(void);

/* 3D solve that allocates nothing. No counterpart in the reference: it exists
 * for callers that cannot call cudaMalloc or hand over a device workspace (a
 * framework that owns all device memory, a latency-critical loop where an
 * allocation would synchronise the device, a foreign-language binding that can
 * only pass the buffers it already owns). Same arguments and results as
 * fteik3d_solve without the workspace: the scratch is a fixed array of
 * FTEIK_NOALLOC_SCRATCH_BYTES compiled into the library, which every GPU that
 * loads the library keeps until exit. Problems whose fteik3d_workspace_bytes()
 * exceed it are rejected with FTEIK_WORKSPACE_TOO_SMALL. All calls on a device
 * share the array (it keeps the last call's contents; the solve clears what
 * must start at zero), so calls that overlap on the GPU race: serialise them.
 * The first call on each device does a one-time set-up with that device
 * current; make it before any stream capture. A cudaDeviceReset may move the
 * array: the next call made outside a stream capture finds it again. Blocking. */
#define FTEIK_NOALLOC_SCRATCH_BYTES (64u << 20)
int fteik3d_solve_noalloc(const double* slow, int nz, int nx, int ny, double dz, double dx,
                          double dy, const double* sources, int nsrc, int nsweep, int grad,
                          double* tt, double* ttgrad, double* vzero, long long spin_limit,
                          void* stream);

/* ------------------------------------------------------------- 3D adjoint --
 * No counterpart in the reference (which is not differentiable): the gradient
 * of a loss on receiver traveltimes with respect to slowness, for tomography.
 *
 * fteik3d_solve_tape runs the same solve as fteik3d_solve (grad = 2: no
 * gradients, branch record kept) and also writes a tape of every change the
 * sweeps make: per node and directional sweep, the code of the operator that
 * changed it (the reference's ttsgn encoding, _fteik3d.py:166-200; 255 =
 * unchanged), and the value each change replaced. A node's first change
 * replaces its initial value (kept for the 8 nodes around the source, Big
 * elsewhere); the values replaced by its next `history` changes go to per-node
 * slots, later ones to an overflow table sized for a quarter of the nodes.
 * `tape` is a device buffer of fteik3d_tape_bytes(nz, nx, ny, nsrc, nsweep,
 * history) bytes: (8 * nsweep + 8 * history + about 4) bytes per node and
 * source, plus each source's set-up. 0 <= history <= 8 * nsweep - 1 (0 when nsweep = 0); with 2 (about
 * 95% of the nodes of layered or gradient models change at most 3 times at
 * nsweep 2) the tape takes 36 bytes per node at nsweep 2, against 144 for a
 * dense record of every sweep. A problem whose changes overflow the table
 * returns FTEIK_TAPE_OVERFLOW (its results are then invalid): retry with a
 * larger history; history = 8 * nsweep - 1 never overflows.
 *
 * fteik3d_adjoint then differentiates exactly the computation that solve ran,
 * sweep by sweep in reverse, so the gradient matches finite differences of
 * the solver for any nsweep, converged or not.
 *  slow, tt, history, tape   the inputs and results of that solve (the tape
 *              also keeps each source's set-up, so the solve's workspace may
 *              be reused once fteik3d_solve_tape returns)
 *  ax0..ax2    device node axes (lengths nz+1, nx+1, ny+1) used for the
 *              receivers' traveltimes (apparent-velocity interpolation)
 *  sources     device [nsrc][3] source coordinates on those axes
 *  receivers   device [nrec][3], the same receivers for every source
 *  grad_tt_rec device [nsrc][nrec] d(loss)/d(traveltime at receiver)
 *  accumulate  0: grad_slow = the sum over these sources; 1: the sum continues
 *              from the values in grad_slow, in the same order, so sources
 *              split into consecutive chunks (each with its own solve and
 *              tape) give the unsplit result bit for bit
 *  grad_slow   device [nz][nx][ny] d(loss)/d(slowness), summed over sources
 *  spin_limit  polls of one progress wait before the reverse pass gives up
 *              with FTEIK_DEVICE_WAIT_TIMEOUT (<= 0: default)
 * The reverse pass undoes every sweep of every source in one persistent
 * launch, as sweeps against the forward direction in the solve's pencil
 * schedule. Deterministic (no floating-point atomics). Both calls block. */
size_t fteik3d_tape_bytes(int nz, int nx, int ny, int nsrc, int nsweep, int history);
int fteik3d_solve_tape(const double* slow, int nz, int nx, int ny, double dz, double dx,
                       double dy, const double* sources, int nsrc, int nsweep, double* tt,
                       double* vzero, void* workspace, size_t workspace_bytes, int history,
                       void* tape, size_t tape_bytes, long long spin_limit, void* stream);
size_t fteik3d_adjoint_workspace_bytes(int nz, int nx, int ny, int nsrc);
int fteik3d_adjoint(const double* slow, int nz, int nx, int ny, double dz, double dx, double dy,
                    int nsrc, int nsweep, const double* tt, int history, const void* tape,
                    size_t tape_bytes, const double* ax0, const double* ax1, const double* ax2,
                    const double* sources, const double* receivers, int nrec,
                    const double* grad_tt_rec, int accumulate, double* grad_slow,
                    void* workspace, size_t workspace_bytes, long long spin_limit, void* stream);
/* fteik3d_adjoint_part: the same reverse pass for the sources src0 ..
 * src0 + nsrc - 1 of a solve of nsrc_tape sources, from that solve's whole tt,
 * tape, sources and grad_tt_rec (all indexed from source 0). Its workspace is
 * fteik3d_adjoint_workspace_bytes(nz, nx, ny, nsrc), for the part only, so a
 * long solve's reverse pass can run in source groups that fit a memory
 * budget; with accumulate = 1 after the first group the result is the
 * whole-solve gradient bit for bit. fteik3d_adjoint is the part src0 = 0,
 * nsrc = nsrc_tape. (No counterpart in the reference.) */
int fteik3d_adjoint_part(const double* slow, int nz, int nx, int ny, double dz, double dx,
                         double dy, int nsrc_tape, int src0, int nsrc, int nsweep,
                         const double* tt, int history, const void* tape, size_t tape_bytes,
                         const double* ax0, const double* ax1, const double* ax2,
                         const double* sources, const double* receivers, int nrec,
                         const double* grad_tt_rec, int accumulate, double* grad_slow,
                         void* workspace, size_t workspace_bytes, long long spin_limit,
                         void* stream);

/* ------------------------------------------------------ model preparation --
 * Replace the SciPy calls of Grid*.resample / Grid*.smooth
 * (fteikpy/_base.py:81-123, 165-212) with device kernels.
 *
 * fteik_resample: RegularGridInterpolator (linear or, with nearest != 0,
 * nearest) at a tensor grid of query points. values: device [dims] (C order,
 * nd = 2 or 3); out: device [out_dims]. The per-axis tables, concatenated
 * axis by axis (out_dims[0] entries, then out_dims[1], ...), are device
 * arrays: idx the lower node index (nearest: the node), y the normalised
 * distance in the cell and ym = 1 - y (both unused for nearest). The corner
 * sum follows scipy's _evaluate_linear order.
 *
 * fteik_correlate1d: out = in correlated with `weights` (device, odd count,
 * centred) along `axis`, mode 'reflect' (scipy.ndimage.correlate1d with
 * origin 0); gaussian_filter is one call per axis. in and out must differ. */
int fteik_resample(int nd, int nearest, const double* values, const int* dims,
                   const int* out_dims, const int* idx, const double* y, const double* ym,
                   double* out, void* stream);
int fteik_correlate1d(int nd, const double* in, const int* dims, int axis,
                      const double* weights, int nweights, double* out, void* stream);

/* ---------------------------------------------------------------- 2D solve --
 * Replaces solve2d / fteik2d / fteik2d_vectorized
 * (fteikpy/_fteik/_fteik2d.py:290-674) as called by Eikonal2D.solve
 * (fteikpy/_solver.py:49-55). Same conventions as the 3D solve with
 * sources HOST [nsrc][2], tt [nsrc][nz+1][nx+1], ttgrad [...][2]. */
size_t fteik2d_workspace_bytes(int nz, int nx, int nsrc, int grad);
int fteik2d_solve(const double* slow, int nz, int nx, double dz, double dx,
                  const double* sources, int nsrc, int nsweep, int grad, double* tt,
                  double* ttgrad, double* vzero, void* workspace, size_t workspace_bytes,
                  void* stream);
/* No counterpart in the reference (a measurement hook): after a 2D solve that
 * ran one warp per source, the node updates of its chains and how many of
 * them took the speculated result (see "sweep2d_speculate"). Blocking. */
int fteik2d_chain_stats(const void* workspace, unsigned long long* nodes,
                        unsigned long long* hits, void* stream);

/* ---------------------------------------------------------- interpolation --
 * interp3d / interp2d (fteikpy/_interp/_interp3d.py:188-195,
 * _interp2d.py:88-95): bi-/tri-linear interpolation of v at query points, as
 * used by Grid*.__call__ (fteikpy/_base.py:56-79,139-163) and by the gradient
 * grids of TraveltimeGrid*.gradient (fteikpy/_grid.py:147-158,267-278).
 *  ax0..ax2  device node axes (ascending), lengths n0..n2
 *  v         device values [n0][n1](n2), element i read at v[i * vstride]
 *  points    device [npts][ndim]
 *  out       device [npts]; fill_value where a point lies outside the axes. */
int fteik_interp3d(const double* ax0, int n0, const double* ax1, int n1, const double* ax2,
                   int n2, const double* v, long long vstride, const double* points, int npts,
                   double fill_value, double* out, void* stream);
int fteik_interp2d(const double* ax0, int n0, const double* ax1, int n1, const double* v,
                   long long vstride, const double* points, int npts, double fill_value,
                   double* out, void* stream);

/* vinterp3d / vinterp2d (fteikpy/_interp/_vinterp3d.py:280-291,
 * _vinterp2d.py:122-131): apparent-velocity traveltime interpolation, as used
 * by TraveltimeGrid*.__call__ (fteikpy/_grid.py:76-101,193-219). Batched: query
 * point p is read from traveltime grid tt + grid_index[p] * tt_stride with
 * source sources[grid_index[p]] and vzero[grid_index[p]]; grid_index may be
 * NULL (all points use grid 0).
 *  sources   device [ngrids][ndim] absolute source coordinates
 *  vzero     device [ngrids] */
int fteik_vinterp3d(const double* ax0, int n0, const double* ax1, int n1, const double* ax2,
                    int n2, const double* tt, long long tt_stride, const int* grid_index,
                    const double* points, int npts, const double* sources, const double* vzero,
                    double fill_value, double* out, void* stream);
int fteik_vinterp2d(const double* ax0, int n0, const double* ax1, int n1, const double* tt,
                    long long tt_stride, const int* grid_index, const double* points, int npts,
                    const double* sources, const double* vzero, double fill_value, double* out,
                    void* stream);

/* ------------------------------------------------------------ ray tracing --
 * ray3d / ray2d (fteikpy/_fteik/_ray3d.py:167-208, _ray2d.py:120-153) as
 * called by TraveltimeGrid*.raytrace (fteikpy/_grid.py:103-145,221-265).
 * Batched: ray r starts at end point ends[r] and walks down the gradient grid
 * ttgrad + grid_index[r] * grad_stride towards sources[grid_index[r]]
 * (grid_index may be NULL: all rays use grid 0).
 *  ttgrad    device [..][nodes][ndim] unit gradient grids
 *  ends      device [nrays][ndim] end points (receivers)
 *  rays      device [nrays][max_step][ndim] scratch output: ray r written end
 *            point first; rays[r][counts[r]] is the source
 *  counts    device [nrays] index of the last point of each ray
 *  status    device [nrays] per-ray FTEIK_* code
 * fteik_ray*_pack then writes the rays source-first (the order ray3d returns)
 * and back to back into packed[sum(counts + 1)][ndim], ray r starting at row
 * offsets[r] (device, exclusive prefix sum of counts + 1). */
int fteik_ray3d(const double* ax0, int n0, const double* ax1, int n1, const double* ax2, int n2,
                const double* ttgrad, long long grad_stride, const int* grid_index,
                const double* ends, int nrays, const double* sources, double stepsize,
                int max_step, int honor_grid, double* rays, int* counts, int* status,
                void* stream);
int fteik_ray2d(const double* ax0, int n0, const double* ax1, int n1, const double* ttgrad,
                long long grad_stride, const int* grid_index, const double* ends, int nrays,
                const double* sources, double stepsize, int max_step, int honor_grid,
                double* rays, int* counts, int* status, void* stream);
int fteik_ray_pack(int ndim, const double* rays, int nrays, int max_step, const int* counts,
                   const long long* offsets, double* packed, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FTEIK_GB300_H */
