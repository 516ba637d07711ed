/*
 * evx.h - C ABI of the GB300 (sm_103a) evoxels time-stepping library (libevx.so).
 *
 * Plain pointers and sizes only.  Field arguments are device pointers to
 * C-contiguous float32 arrays of shape (Nx, Ny, Nz), z fastest - one channel
 * of the reference's (C, Nx, Ny, Nz) torch layout (evoxels/voxelgrid.py:126-130).
 * Every call is stream-ordered on the cudaStream_t it is given (passed as
 * void*; NULL = legacy default stream) and returns an int status (EVX_OK = 0);
 * evx_last_error() gives the message of the last failure on the calling
 * thread.  No C++ exception crosses this boundary.  Calls never mutate their
 * input fields (the reference's steps are functional: evoxels/solvers.py:204).
 *
 * Workspaces are caller-allocated device memory; the library allocates no
 * device memory of its own except inside evx_ch_plan_create (k^2 tables).
 */
#ifndef EVX_H
#define EVX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define EVX_OK               0
#define EVX_ERR_BAD_SHAPE    1  /* reference: ValueError (evoxels/boundary_conditions.py:76-82) */
#define EVX_ERR_BAD_ARG      2
#define EVX_ERR_BAD_BC       3  /* reference: ValueError (evoxels/problem_definition.py:67-102) */
#define EVX_ERR_CUFFT        4
#define EVX_ERR_CUDA         5
#define EVX_ERR_NONFINITE    6  /* reference: NaN abort (evoxels/solvers.py:163-165) */
#define EVX_ERR_TOO_LARGE    7
#define EVX_ERR_WORKSPACE    8
#define EVX_ERR_UNSUPPORTED  9  /* reference: NotImplementedError (evoxels/problem_definition.py:151-155) */

/* ---- boundary conditions (evoxels/boundary_conditions.py:9-59) --------- */
#define EVX_BC_PERIODIC   0
#define EVX_BC_NEUMANN    1   /* ghost = first/last interior value */
#define EVX_BC_DIRICHLET  2   /* ghost = 2*v - first/last interior value */

typedef struct evx_bc {
    int32_t kind[3];      /* x, y, z */
    float   two_v_lo[3];  /* float32(2.0*v_left)  of Dirichlet axes (0 otherwise) */
    float   two_v_hi[3];  /* float32(2.0*v_right) of Dirichlet axes (0 otherwise) */
} evx_bc;

/* Grid geometry: shape, the spacing as the reference's python doubles
 * (VoxelFields.spacing, evoxels/voxelfields.py:84-86; used for the k-grid),
 * and the float32 div_dx / div_dx2 factors (evoxels/voxelgrid.py:29-30) with
 * float32 sum(div_dx2) (evoxels/fd_stencils.py:74) used by the stencils. */
typedef struct evx_grid {
    int32_t nx, ny, nz, reserved;
    double  h[3];
    float   inv_h[3];
    float   inv_h2[3];
    float   inv_h2_sum;
} evx_grid;

/* Cahn-Hilliard parameters (evoxels/problem_definition.py:290-305), each the
 * float32 rounding of the python-double expression the reference evaluates:
 *   D        = D
 *   kappa    = 2*eps                      (gradient coefficient, mu = mu_hom - kappa*lap)
 *   w        = 18/eps by default          (bulk coefficient, below)
 *   A        = A (0.25)
 *   sym_coef = -2*eps*D*A                 (fourier_symbol = sym_coef*(k^2)^2)
 *   dt       = dt                         (prefac = dt/(1 - dt*symbol), evoxels/timesteppers.py:77)
 *   bulk     = form of the homogeneous chemical potential mu_hom(c):
 *              EVX_BULK_DOUBLE_WELL  w*c*(1-c)*(1-2c)   (the default, evoxels/problem_definition.py:305)
 *              EVX_BULK_REGULAR_SOLUTION  log(c) - log(1-c) + w*(1-2c)   (the logarithmic free
 *              energy the reference passes as a callable, docs/notebooks/01-using-solvers.ipynb;
 *              forward steps only) */
#define EVX_BULK_DOUBLE_WELL       0
#define EVX_BULK_REGULAR_SOLUTION  1
typedef struct evx_ch_params {
    float D, kappa, w, A, sym_coef, dt;
    int32_t bulk;
} evx_ch_params;

/* Two-phase Allen-Cahn parameters (evoxels/problem_definition.py:374-447), the
 * float32 roundings of the python-double values the reference uses:
 *   w = 18/eps by default (potential w*c*(1-c)*(1-2c)), eps, gab, M, force,
 *   three_over_eps = 3/eps, curvature, one_minus_curvature = 1 - curvature. */
typedef struct evx_ac_params {
    float w, eps, gab, M, force, three_over_eps, curvature, one_minus_curvature;
} evx_ac_params;

/* ---- library info -------------------------------------------------------- */
const char* evx_last_error(void);
int evx_version(void);

/* Host-only: per-axis k^2 tables exactly as VoxelGrid.rfft_k_squared builds
 * them in float32 (evoxels/voxelgrid.py:84-90,110-114): kx2[nx], ky2[ny],
 * kz2[nz/2+1]; k^2(i,j,k) = (kx2[i] + ky2[j]) + kz2[k].  Needs no GPU. */
int evx_k2_tables_host(int nx, int ny, int nz, double hx, double hy, double hz,
                       float* kx2, float* ky2, float* kz2);

/* ---- finite-difference stencil path ------------------------------------- */

/* ReactionDiffusion.rhs with f = 0: r = D*laplace(pad_bc(u))
 * (evoxels/problem_definition.py:226-229, evoxels/fd_stencils.py:62-75). */
int evx_rd_rhs(const float* u, float* r, const evx_grid* g, const evx_bc* bc,
               float D, void* stream);

/* nsteps ForwardEuler steps of ReactionDiffusion (f = 0):
 * u <- u + dt*(D*laplace(pad_bc(u)) + 0)   (evoxels/timesteppers.py:42-43).
 * u_in is read only; the result lands in u_out.  scratch: one field
 * (Nx*Ny*Nz floats) used as the ping-pong buffer when nsteps > 1 (may be
 * NULL when nsteps == 1).  steps_per_pass in {1,2,4} selects temporal
 * blocking (results are bit-identical for every choice). */
int evx_fd_forward(const float* u_in, float* u_out, float* scratch,
                   const evx_grid* g, const evx_bc* bc, float D, float dt,
                   int nsteps, int steps_per_pass, void* stream);

/* Allocation-free variant of evx_fd_forward (no counterpart in the reference):
 * for callers that cannot let a library allocate device memory, such as hosts
 * whose device memory comes only from their own pre-reserved pool, or
 * bindings passing buffers from a foreign allocator.  The ping-pong scratch
 * lives in a static device array of EVX_FD_NOALLOC_MAX_VOXELS floats (16 MiB),
 * held on every GPU that loads the library until the process exits; larger
 * grids are rejected with EVX_ERR_TOO_LARGE.  The first call on a device looks
 * up the array's device address, so make that first call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race.
 * Calls no cudaMalloc, cudaFree or allocating library routine. */
#define EVX_FD_NOALLOC_MAX_VOXELS (1u << 22)
int evx_fd_forward_noalloc(const float* u_in, float* u_out, const evx_grid* g, const evx_bc* bc,
                           float D, float dt, int nsteps, int steps_per_pass, void* stream);

/* Adjoint of evx_fd_forward with respect to u_in: lam_out = (dU_n/dU_0)^T lam_in.
 * The transposed stencil uses homogeneous ghosts (a Dirichlet ghost 2v-u0
 * contributes -1*u0, a Neumann ghost +1*u0).  scratch as above. */
int evx_fd_adjoint(const float* lam_in, float* lam_out, float* scratch,
                   const evx_grid* g, const evx_bc* bc, float D, float dt,
                   int nsteps, void* stream);

/* ForwardEuler update out = u + dt*r (evoxels/timesteppers.py:43) for a
 * precomputed right-hand side, n elements. */
int evx_fe_update(const float* u, const float* r, float dt, float* out, size_t n, void* stream);

/* ---- Cahn-Hilliard path ---------------------------------------------------- */

/* TwoPhaseAllenCahn.rhs (evoxels/problem_definition.py:420-447) for any BC:
 * clip, double-well potential, curvature-weighted 7-point Laplacian plus the
 * 19-point normal Laplacian (evoxels/fd_stencils.py:77-103), bit-identical to
 * the reference's float32 arithmetic.  u and r: (nx, ny, nz) float32. */
int evx_ac_rhs(const float* u, float* r, const evx_grid* g, const evx_bc* bc,
               const evx_ac_params* p, void* stream);
/* The same rhs of a Runge-Kutta stage input, r = rhs(u + c*k), the stage field
 * formed on the fly as evx_fe_update forms it (float32(c), one rounding per
 * operation), so RungeKutta4's k2..k4 equal rhs(evx_fe_update(u, k, c)) bit for
 * bit without the stage field in HBM. */
int evx_ac_rhs_stage(const float* u, const float* k, float c, float* r, const evx_grid* g,
                     const evx_bc* bc, const evx_ac_params* p, void* stream);

/* RungeKutta4.step's combination (evoxels/timesteppers.py:61):
 * out = u + dt6*(((k1 + 2*k2) + 2*k3) + k4), dt6 = float32(dt/6); the stage
 * inputs u + c*k are evx_fe_update. */
int evx_rk4_combine(const float* u, const float* k1, const float* k2, const float* k3, const float* k4,
                    float dt6, float* out, size_t n, void* stream);

/* One Runge-Kutta-Chebyshev stage coefficient set (float32, as the reference's
 * tensors hold them): mu0[j], nu[j], (1 - mu0[j]) - nu[j], mu1[j]*dt and, for
 * RKC2, gamma[j]*dt (evoxels/timesteppers.py:219-229, 263-280). */
typedef struct evx_rkc_coeffs {
    float mu0, nu, one_minus_mu0_nu, mu1_dt, gamma_dt;
} evx_rkc_coeffs;

/* RKC1.step / RKC2.step stage recursion (evoxels/timesteppers.py:237-243,
 * 286-294): out = mu0*y_curr + nu*y_prev + (1-mu0-nu)*u + mu1*dt*r
 * [+ gamma*dt*r0], summed left to right, each product rounded.  r0 = NULL
 * drops the last term (RKC1).  The first stage u + mu11*dt*rhs(u) is
 * evx_fe_update. */
int evx_rkc_stage(const float* u, const float* y_curr, const float* y_prev, const float* r, const float* r0,
                  const evx_rkc_coeffs* c, float* out, size_t n, void* stream);

/* CahnHilliard.rhs (evoxels/problem_definition.py:328-371) for any BC. */
int evx_ch_rhs(const float* u, float* r, const evx_grid* g, const evx_bc* bc,
               const evx_ch_params* p, void* stream);

typedef struct evx_ch_plan evx_ch_plan;

/* Plan for the periodic pseudo-spectral IMEX step (evoxels/timesteppers.py:64-89)
 * on an (nx, ny, nz) grid: cuFFT R2C/C2R plans without auto-allocated work
 * areas, and the k^2 tables.  flags: bit 0 = also build the batch-2 C2R plan
 * used by parameter gradients; bit 1 = always use cuFFT's 3-D transforms (by
 * default a power-of-two nx uses cuFFT over (y, z) and a fused x-pass that
 * does the x transforms and the k-space multiply in one read and write). */
int evx_ch_plan_create(evx_ch_plan** plan, const evx_grid* g, int flags);
/* Same for a problem with boundary conditions bc (NULL = periodic): y and z
 * periodic, x periodic, Neumann or Dirichlet.  A non-periodic x axis runs the
 * reference's mirrored step (evoxels/boundary_conditions.py:64-70,
 * evoxels/voxelgrid.py:116-124, evoxels/timesteppers.py:85-89): the rhs with the
 * BC ghosts, extended along x by its mirror image (Neumann) or the negated
 * mirror image (Dirichlet) to 2*nx, transformed with the 2*nx-point k-grid,
 * and trimmed back to nx.  Power-of-two nx <= 256 do the extension inside the
 * x-pass (no extra HBM traffic); others run cuFFT over (2*nx, ny, nz).  The
 * adjoint and stored spectra are not built for it (EVX_ERR_UNSUPPORTED);
 * otherwise EVX_ERR_BAD_BC as the reference's verify_fft_bc_config
 * (evoxels/problem_definition.py:138-167). */
int evx_ch_plan_create_bc(evx_ch_plan** plan, const evx_grid* g, const evx_bc* bc, int flags);
/* flags bit 2: with the x-pass and ny, nz in {64, 128, 256}, use the fused
 * (y, z) kernels (evx_fft_yz_r2c/c2r) instead of cuFFT's (y, z) plans.  Off by
 * default: on GB300 at 256^3 they take 55/68 us per transform against cuFFT's
 * 64/61 us (the C2R is latency-bound on its distributed-shared-memory gathers).
 * By default an x-pass plan with nz = 256 keeps the half spectrum y-contiguous,
 * (nx, nz/2+1, ny): the z pass is evx_fft_z_r2c/c2r and the y transform one
 * contiguous batched cuFFT C2C (56/61 us per transform at 256^3 against
 * 64/61 us; for nz = 32, 64 it is slower than cuFFT's plans, for 128 even).
 * flags bit 4: the same for nz in {32, 64, 128}; bit 3: cuFFT's 2-D (y, z)
 * plans for every nz.  The same bits apply to evx_batch_create. */
int evx_ch_plan_destroy(evx_ch_plan* plan);

/* Bytes of device workspace (256-byte aligned start) the plan's calls need. */
size_t evx_ch_workspace_bytes(const evx_ch_plan* plan);

/* ExponentialEuler.step's spectral update (evoxels/timesteppers.py:195-199)
 * for any rhs on the plan's grid: out = u + irfftn(mult * rfftn(pad_fft(r)))[:nx],
 * pad_fft the plan's x extension (evoxels/boundary_conditions.py:61-71).  mult is
 * the real multiplier table dt*phi1(dt*symbol) over the (extended) rfft grid,
 * float32 on the device, in the plan's spectrum order (evx_ch_mult_layout):
 * [nxe][ny][nz/2+1], or [nxe][nz/2+1][ny] for the plans whose z pass keeps y
 * contiguous.  r and u are read only. */
int evx_spectral_update(evx_ch_plan* plan, const float* u, const float* r, const float* mult, float* out,
                        void* workspace, void* stream);

/* Layout of the multiplier tables of evx_spectral_update and
 * evx_ch_forward_mult on this plan: 0 [nxe][ny][nz/2+1] (the rfftn order),
 * 1 [nxe][nz/2+1][ny]; -1 for a NULL plan. */
int evx_ch_mult_layout(const evx_ch_plan* plan);

/* nsteps ExponentialEuler steps of CahnHilliard in one call, the update fused
 * into the next step's rhs pass as in evx_ch_forward: each step is
 * u + irfftn(mult * rfftn(pad_fft(rhs(u))))[:nx] with the CahnHilliard rhs of
 * prm (prm->dt is not used), bit-identical to nsteps evx_ch_rhs +
 * evx_spectral_update calls.  nonfinite as in evx_ch_forward. */
int evx_ch_forward_mult(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps, const float* mult,
                        const evx_ch_params* prm, int* nonfinite, void* workspace, void* stream);

/* One PseudoSpectralIMEX step of CahnHilliard (evoxels/timesteppers.py:85-89):
 * u_out = u_in + irfftn(prefac * rfftn(rhs(u_in))).  u_in is read only. */
int evx_ch_step(evx_ch_plan* plan, const float* u_in, float* u_out,
                const evx_ch_params* p, void* workspace, void* stream);

/* nsteps IMEX steps, the update of each step fused into the next step's rhs
 * pass.  traj (optional, NULL for none) receives states u_1..u_n as nsteps
 * consecutive fields; u_out receives u_n.  nonfinite (optional device int)
 * is set to 1 if the final state holds a NaN or Inf. */
int evx_ch_forward(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps,
                   float* traj, const evx_ch_params* p, int* nonfinite,
                   void* workspace, void* stream);

/* Adjoint of nsteps IMEX steps.  states: nsteps+1 consecutive fields u_0..u_n
 * of the forward trajectory; lam_in = dL/du_n; lam_out = dL/du_0.
 * grads (optional device double[3]) accumulates dL/dD, dL/dkappa, dL/dw
 * (kappa, w as in evx_ch_params; needs a plan made with flags bit 0).
 * lam_in is read only; lam_in and lam_out must be 16-byte aligned (they feed
 * cuFFT R2C).  A plan of evx_ch_plan_create_bc with a Neumann or Dirichlet
 * x axis (the mirrored-x step, evoxels/boundary_conditions.py:64-70) gives the
 * adjoint of that step; its grads need no flags bit 0, and it keeps no stored
 * spectra (evx_ch_adjoint_spectra with spectra = NULL). */
int evx_ch_adjoint(evx_ch_plan* plan, const float* states, int nsteps,
                   const float* lam_in, float* lam_out, const evx_ch_params* p,
                   double* grads, void* workspace, void* stream);

/* Stored increment spectra (no reference counterpart: they serve the adjoint).
 * Floats per step of the spectrum dU = prefac/N * rfftn(rhs) whose inverse
 * transform is u_{s+1} - u_s, in the x-pass's internal element order; 0 when
 * the plan has no x-pass (nx not a power of two in [8, 512], or flags bit 1). */
size_t evx_ch_spectrum_floats(const evx_ch_plan* plan);

/* evx_ch_forward that also writes step s's increment spectrum to
 * spectra + s*evx_ch_spectrum_floats(plan) (spectra: 16-byte aligned, nsteps
 * spectra; NULL = plain evx_ch_forward).  EVX_ERR_UNSUPPORTED without x-pass. */
int evx_ch_forward_spectra(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps,
                           float* traj, float* spectra, const evx_ch_params* p, int* nonfinite,
                           void* workspace, void* stream);

/* evx_ch_adjoint with the spectra evx_ch_forward_spectra stored for the same
 * states and parameters.  With grads, the two mobility sums are formed by
 * Parseval in the adjoint x-pass, so each step needs one inverse transform
 * (not two) and the pullback reads neither u_{s+1} nor a second field; the
 * plan needs no flags bit 0.  states: u_0..u_{n-1} are read (u_n is not).
 * spectra NULL or grads NULL: same as evx_ch_adjoint. */
int evx_ch_adjoint_spectra(evx_ch_plan* plan, const float* states, const float* spectra, int nsteps,
                           const float* lam_in, float* lam_out, const evx_ch_params* p,
                           double* grads, void* workspace, void* stream);

/* Fused 2-D (y, z) real-to-complex / complex-to-real transforms of the nx
 * planes of a float32 (nx, ny, nz) field, in cuFFT's batched 2-D layout and
 * scaling (spec (nx, ny, nz/2+1) complex64 as interleaved floats, unnormalised);
 * one HBM pass each (thread-block clusters exchange the transposed data in
 * distributed shared memory).  ny, nz in {64, 128, 256}; else
 * EVX_ERR_UNSUPPORTED.  No reference counterpart: building blocks of the
 * spectral step exposed for tests and other hosts. */
int evx_fft_yz_r2c(const float* in, float* spec, int nx, int ny, int nz, void* stream);
int evx_fft_yz_c2r(const float* spec, float* out, int nx, int ny, int nz, void* stream);

/* Real transforms along z of every (x, y) row with a y-contiguous half
 * spectrum: R2C reads in[x][y][z] and writes spec[x][kz][y], kz in [0, nz/2]
 * (cuFFT's unnormalised values); C2R reads spec[x][kz][y] (imaginary parts of
 * kz = 0 and nz/2 ignored) and writes out[x][y][z].  nz in {32, 64, 128, 256}, else
 * EVX_ERR_UNSUPPORTED.  The z pass of the x-pass plans (the y transform is then
 * one contiguous batched C2C); no reference counterpart. */
int evx_fft_z_r2c(const float* in, float* spec, int nx, int ny, int nz, void* stream);
int evx_fft_z_c2r(const float* spec, float* out, int nx, int ny, int nz, void* stream);

/* Device-side status bits, synchronous read (reset != 0 clears them): bit 0 =
 * a bounded wait of the pipelined x-pass on its tile loads gave up (the
 * results of that call are invalid).  Returns -1 if the read itself failed. */
int evx_device_status(int reset);

/* Queue a copy of the device status word into dst (host-pinned or device
 * memory) on the given stream, ordered after the work queued there before it; the
 * asynchronous form of evx_device_status for loops that must not stall the
 * device (a frame pipeline reads it with the frame's data). */
int evx_device_status_async(int* dst, void* stream);

/* Poll limit of the x-pass's bounded waits on its tile loads on the current
 * device (default 2^22 when polls < 0).  A call whose wait runs out sets bit
 * 0 of the device status, stops storing results and returns once its loads in
 * flight have landed.  A limit of 0 makes every such wait give up at once,
 * which exercises that path without any fault. */
int evx_set_wait_polls(int polls);

/* Tile shape of the periodic fast-path stencil kernels (single grids):
 * -1 automatic (32x32 when nz is a multiple of 32 but not of 64, else 16x64),
 * 0 = 16x64, 1 = 32x32.  Results are bit-identical for every choice.  A
 * change drops the plans' captured step graphs. */
int evx_set_tile_variant(int variant);

/* ---- batched uneven instances ---------------------------------------------
 * Many independent periodic Cahn-Hilliard grids of different sizes stepped
 * together (the reference batches parameter-estimation solves with jax.vmap,
 * evoxels/inversion.py:121, over grids of one shape).  Fields of all instances
 * live in one packed float32 buffer of evx_batch_field_floats() floats;
 * instance i occupies [offsets[i], offsets[i] + nx*ny*nz) (evx_batch_offsets).
 * Each instance needs nz % 4 == 0. */
typedef struct evx_batch evx_batch;

typedef struct evx_batch_instance {
    int32_t nx, ny, nz, reserved;
    double  h[3];
    float   inv_h[3], inv_h2[3], inv_h2_sum;
    evx_ch_params params;
} evx_batch_instance;

typedef struct evx_batch_tuning {
    int32_t tile_variant;    /* -1 automatic per instance, 0 = 16x64, 1 = 32x32 */
    int32_t x_chunk;         /* x planes per work item (0 = automatic) */
    int32_t blocks_per_sm;   /* persistent blocks per SM (0 = occupancy limit) */
    int32_t fft_group_max;   /* instances per cuFFT plan (0 = whole shape group) */
    int32_t graph_steps;     /* fused steps per captured CUDA graph (0 = no graph) */
} evx_batch_tuning;

int evx_batch_create(evx_batch** batch, const evx_batch_instance* inst, int n,
                     const evx_batch_tuning* tuning, int flags);
int evx_batch_destroy(evx_batch* batch);
size_t evx_batch_field_floats(const evx_batch* batch);
size_t evx_batch_workspace_bytes(const evx_batch* batch);
int evx_batch_work_items(const evx_batch* batch);
int evx_batch_offsets(const evx_batch* batch, int64_t* offsets);

/* nsteps IMEX steps of every instance (as evx_ch_forward, on packed buffers). */
int evx_batch_forward(evx_batch* batch, const float* u_in, float* u_out, int nsteps,
                      float* traj, int* nonfinite, void* workspace, void* stream);

/* Adjoint of nsteps steps of every instance (as evx_ch_adjoint); grads
 * (optional, device double[3*n]) accumulates dL/dD, dL/dkappa, dL/dw per
 * instance, in the caller's instance order. */
int evx_batch_adjoint(evx_batch* batch, const float* states, int nsteps,
                      const float* lam_in, float* lam_out, double* grads,
                      void* workspace, void* stream);

/* Floats of one step's stored increment spectra for all instances (the
 * x-pass layout for power-of-two groups, the rfftn layout for the others). */
size_t evx_batch_spectrum_floats(const evx_batch* batch);

/* evx_batch_forward with the trajectory and, in spectra (16-byte aligned,
 * nsteps * evx_batch_spectrum_floats floats), each step's increment spectra. */
int evx_batch_forward_spectra(evx_batch* batch, const float* u_in, float* u_out, int nsteps,
                              float* traj, float* spectra, int* nonfinite, void* workspace,
                              void* stream);

/* evx_batch_adjoint with the stored spectra of the same steps: the mobility
 * gradient sums by Parseval in k-space (no inverse transform of the second
 * adjoint field, no h or u_{s+1} reads in the pullback).  lam_out equals
 * evx_batch_adjoint's bit for bit; the gradients agree to float32 rounding. */
int evx_batch_adjoint_spectra(evx_batch* batch, const float* states, const float* spectra,
                              int nsteps, const float* lam_in, float* lam_out, double* grads,
                              void* workspace, void* stream);

/* ---- inversion loss ---------------------------------------------------------- */

/* loss = mean((u - target)^2) (device double) and, if lam != NULL, its gradient
 * lam = 2*(u - target)/n: the seed of the adjoint for the parameter-estimation
 * workflow (evoxels/inversion.py:105-124 fits simulated to observed fields).
 * scratch: evx_mse_scratch_bytes(n) bytes of device memory for partial sums. */
size_t evx_mse_scratch_bytes(size_t n);

/* The solver's frame check (evoxels/solvers.py:163-165) on the device:
 * *flag (device int) = 1 if any of the n floats at x is NaN, else 0. */
int evx_nan_flag(const float* x, size_t n, int* flag, void* stream);
int evx_mse_grad(const float* u, const float* target, size_t n, float* lam, double* loss,
                 void* scratch, size_t scratch_bytes, void* stream);

/* ---- instrumentation ------------------------------------------------------ */

/* Per-kernel timing: when enabled, every kernel launch and cuFFT execution of
 * the library is bracketed by CUDA events on its stream.  collect() waits for
 * them and accumulates milliseconds per named slot; query() walks the slots
 * (returns -1 past the last).  Off by default. */
void evx_prof_enable(int on);
int evx_prof_collect(void);
void evx_prof_reset(void);
int evx_prof_query(int index, char* name, int name_cap, double* total_ms, long long* count);

/* Number of this library's own kernel launches since load (cuFFT's excluded;
 * a replayed graph counts its kernels once per replay). */
unsigned long long evx_launch_count(void);

/* CUDA graph replay of repeated multi-step calls (evx_ch_forward*,
 * evx_ch_adjoint*, evx_batch_forward/adjoint): a plan runs the first call
 * with a given set of pointers, step count and parameters eagerly, captures
 * the second into a graph and replays that graph for later identical calls
 * (bit-identical results; at most 4 graphs kept per plan).  Calls made while
 * the stream is being captured by the caller, or with kernel timing on, run
 * eagerly.  On by default; EVX_GRAPHS=0 in the environment or
 * evx_set_graphs(0) turns it off. */
void evx_set_graphs(int on);
int evx_graphs_enabled(void);

#ifdef __cplusplus
}
#endif

#endif /* EVX_H */
