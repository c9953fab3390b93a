/*
 * libglgpu: GB300-native (sm_103a) 2D Ginzburg-Landau hot path behind a C ABI.
 *
 * Replaces the kernels that microsoft/svirl compiles at run time and looks up by
 * name (svirl/parallel/startup.py:74-82, Startup.get_function), together with the
 * host loops that drive them (svirl/solvers/td.py, svirl/solvers/cg.py,
 * svirl/observables/observables.py).  Plain pointers and sizes only.
 *
 * Conventions
 *  - dtype 4 = float32 (complex64 psi), 8 = float64 (complex128 psi), as the
 *    reference's GLSolver(dtype=...) (svirl/__init__.py:65-71).
 *  - Host buffers use the reference's flat layouts (svirl/storage/arrays.py:327-365):
 *      psi: N = Nx*Ny complex values, n = i + Nx*j, interleaved (re, im);
 *      A:   Nab reals, [a (i + (Nx-1)*j) | b (Na + i + Nx*j)];
 *      material tiling: Nc = (Nx-1)*(Ny-1) bytes, cell i + (Nx-1)*j, 0 = not
 *      superconducting; NULL = whole domain.
 *  - Every call is synchronous with respect to the host unless stated otherwise,
 *    runs on the handle's own CUDA stream, and returns GLGPU_OK (0) or a
 *    negative GLGPU_E_* code; glgpu_last_error() gives the message.
 *  - Device state is owned by the handle; caller buffers are copied.  The state
 *    get/set calls accept host or device pointers (unified addressing).  One
 *    handle per host thread (thread-compatible, not thread-safe).
 */
#ifndef GLGPU_H
#define GLGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLGPU_OK 0
#define GLGPU_E_ARG (-1)      /* bad argument (sizes, dtype, NULL) */
#define GLGPU_E_CUDA (-2)     /* CUDA runtime error */
#define GLGPU_E_OOM (-3)      /* device allocation failed */
#define GLGPU_E_TIMEOUT (-4)  /* a device loop hit its iteration guard */
#define GLGPU_E_NAN (-5)      /* NaN residual seen (state still updated like the reference) */
#define GLGPU_E_NOROOT (-6)   /* no real non-negative line-search root */

typedef struct glgpu_handle glgpu_handle;

/* Geometry and precision: svirl/__init__.py:73-117 (Nx, Ny >= 4). */
typedef struct {
    int32_t Nx, Ny;
    double dx, dy;
    int32_t dtype;
} glgpu_grid;

/* Parameters: svirl/vars/params.py:47-118,270-325 and the stop criteria of
 * svirl/__init__.py:147-151.  kappa <= 0 or inf means kappa = inf (A fixed). */
typedef struct {
    double kappa;           /* gl_parameter */
    double sigma;           /* normal_conductivity */
    double epsilon;         /* linear_coefficient (scalar) */
    double H;               /* homogeneous_external_field */
    double stop_psi;        /* stop_criterion_order_parameter (clamped like svirl/solvers/td.py:52-66) */
    double stop_A;          /* stop_criterion_vector_potential */
    double langevin_psi;    /* order_parameter_Langevin_coefficient */
    double langevin_A;      /* vector_potential_Langevin_coefficient */
    uint32_t rand_t;        /* Langevin time seed, svirl/solvers/td.py:35-37 */
    int32_t pad_;
} glgpu_params;

/* Per-call TDGL statistics. */
typedef struct {
    int32_t steps;
    int32_t max_sweeps_psi, max_sweeps_A;
    int32_t last_sweeps_psi, last_sweeps_A;
    int32_t nan_seen;
    int64_t total_sweeps_psi, total_sweeps_A;
    uint32_t rand_t;        /* Langevin seed after the call */
    int32_t used_graph;     /* 1: device-side loop (CUDA graph), 0: host-driven loop */
    int64_t sweep_launches; /* Jacobi sweep kernel launches (psi and A) */
} glgpu_td_stats;

/* --- lifetime: GLSolver construction / destruction (svirl/__init__.py:30-179,
 *     svirl/parallel/startup.py:17-71) */
int glgpu_create(const glgpu_grid* grid, int32_t device, glgpu_handle** out);
int glgpu_destroy(glgpu_handle* h);
const char* glgpu_last_error(const glgpu_handle* h);   /* h may be NULL: last create error */
int glgpu_version(void);
/* Jacobi sweeps of the psi step done by one launch of the psi sweep kernel
 * (temporal blocking; every sweep is still written, so the loop stops exactly
 * where the reference's one-sweep-per-launch loop stops). */
int glgpu_psi_sweeps_per_launch(void);
/* Rows per warp strip of the psi sweep chosen for this handle (from the compiled
 * strip heights, by the item-count model of the persistent sweep); 0 if h is NULL. */
int glgpu_psi_strip_rows(const glgpu_handle* h);
/* Force the strip height (one of the compiled heights; 0 = the model's choice).
 * Results do not depend on it: every node gets the same arithmetic. */
int glgpu_set_psi_strip_rows(glgpu_handle* h, int32_t rows);
/* The FP32 psi sweep kernel: 0 (default) = the register-strip kernel (the FP64
 * build always uses it); 1 = inputs staged in shared memory by bulk copies
 * (TMA), four strips per CTA, measured slower on GB300 (172 against 89 us per
 * launch on the 2049^2 workload).  Both compute the same values bitwise. */
int glgpu_set_psi_sweep_kernel(glgpu_handle* h, int32_t select);
/* Time stepping of the order parameter: 0 (default) = backward Euler, the
 * reference's scheme (svirl/cuda/td.h:4-133); 1 = Crank-Nicolson of the
 * reference's commented-out kernel (iterate_order_parameter_jacobi_step_CN,
 * svirl/cuda/td.h:136-292, which no host code of the reference launches) with
 * the explicit half of every link from the step's start (the trapezoidal rule);
 * 2 = that kernel exactly as written (the explicit half of three links from the
 * current iterate, which counts them twice).  Same Jacobi loop and stop rule
 * (on the squared change, as the kernel computes it).  Single handles only
 * (glgpu_batch_td rejects them). */
int glgpu_set_psi_scheme(glgpu_handle* h, int32_t scheme);

/* --- fixed vortices (svirl/vars/fixed_vortices.py, svirl/solvers/td.py:120-154,
 *     204-216, 252-325): the irregular vector potential A_irr (Nab values, flat
 *     [a | b], or NULL to remove it) and the phase-lock node list (flat node
 *     indices; count 0 removes it).  The TD step adds A_irr to the first N elements
 *     of A around the psi loop and A to the first N elements of A_irr around the A
 *     loop, as the reference does, so the device copy of A_irr changes during A
 *     loops: the getter returns it.  With td_copy_only the setter only replaces
 *     the values of an A_irr already set (resuming from a checkpoint). */
int glgpu_set_irregular_vector_potential(glgpu_handle* h, const void* vpi, int32_t td_copy_only);
int glgpu_get_irregular_vector_potential(glgpu_handle* h, void* out);
int glgpu_set_phase_lock(glgpu_handle* h, const int32_t* nodes, int32_t count);

/* --- state and parameters (svirl/vars/vars.py:53-127, svirl/vars/params.py,
 *     svirl/mesh/grid.py:102-127) */
int glgpu_set_params(glgpu_handle* h, const glgpu_params* p);
int glgpu_get_params(const glgpu_handle* h, glgpu_params* p);
int glgpu_set_order_parameter(glgpu_handle* h, const void* psi);
int glgpu_get_order_parameter(glgpu_handle* h, void* psi);
int glgpu_set_vector_potential(glgpu_handle* h, const void* ab);
int glgpu_get_vector_potential(glgpu_handle* h, void* ab);
int glgpu_set_external_vector_potential(glgpu_handle* h, const void* abei);  /* NULL clears */
int glgpu_set_material_tiling(glgpu_handle* h, const uint8_t* mt);          /* NULL = full domain */
int glgpu_set_linear_coefficient_field(glgpu_handle* h, const void* eps);   /* N reals or NULL */

/* --- TDGL: TD._solve (svirl/solvers/td.py:342-377); kernels
 *     iterate_order_parameter_jacobi_step (svirl/cuda/td.h:4-133) and
 *     iterate_vector_potential_jacobi_step (svirl/cuda/td.h:310-463).
 *     eqn: 0 = both (td.py:342), 1 = order parameter only (td.py:337),
 *     2 = vector potential only (td.py:444). */
int glgpu_td(glgpu_handle* h, double dt, int32_t Nt, int32_t eqn, glgpu_td_stats* stats);
int glgpu_set_use_graphs(glgpu_handle* h, int32_t enable);
/* Safety net of the device-side Jacobi loops: a loop that has launched this many
 * sweep kernels without meeting the stop rule ends, and the call returns
 * GLGPU_E_TIMEOUT; a time step whose loop was cut keeps the state it started
 * from (its sweeps are discarded).  0 (the default) = 1088 launches, above the
 * reference's cap of 1024 sweeps per step (svirl/solvers/td.py:164,274), which
 * the loop also applies, so by default the guard fires only if that cap fails.
 * The reference's host loop has no guard. */
int glgpu_set_loop_guard(glgpu_handle* h, int32_t launches);

/* --- timing (CUDA events on the handle's stream; no counterpart in the reference,
 *     which has no timing code: its profiler calls are commented out,
 *     svirl/solvers/cg.py:473,546):
 *   glgpu_td_timed:    glgpu_td, plus the device time of the whole TD run;
 *   glgpu_time_sweeps: average device time of one Jacobi sweep kernel launch
 *                      (which 0 = psi; 1 = A, timed as pairs of sweeps 0 and 1,
 *                      since the second of a pair reuses the first's link terms),
 *                      L2 flushed before each launch (A: before each pair);
 *                      leaves the state at rest unchanged. */
int glgpu_td_timed(glgpu_handle* h, double dt, int32_t Nt, int32_t eqn, glgpu_td_stats* stats, double* elapsed_ms);
int glgpu_time_sweeps(glgpu_handle* h, int32_t which, int32_t nrep, double* avg_ms);

/* --- observables (svirl/observables/observables.py:29-149) */
int glgpu_free_energy(glgpu_handle* h, double* energy);          /* free_energy_pseudodensity + gsum, observables.h:250-362 */
int glgpu_magnetic_field(glgpu_handle* h, void* B);              /* Nc reals, observables.h:4-37 */
int glgpu_current_density(glgpu_handle* h, void* j);             /* Nab reals, observables.h:40-156 (kappa=inf: supercurrent) */
int glgpu_supercurrent_density(glgpu_handle* h, void* js);       /* Nab reals, observables.h:159-235 */

/* --- vortex detector (svirl/observables/vortex_detector.py:31-72): plaquette
 *     winding scan on the GPU with a relaxed predicate; for each candidate cell
 *     (sorted by cell index) `corners` receives 4 psi values (00, p0, pp, 0p;
 *     complex in dtype) and 4 link values (a00, a0p, b00, bp0; dtype), so that
 *     the caller can apply the reference's exact predicate and triangulation. */
int glgpu_vortex_candidates(glgpu_handle* h, int32_t cap, int32_t* n_out, int32_t* cells, void* corners);

/* --- modified nonlinear CG, one iteration in phases (svirl/solvers/cg.py:238-551):
 *   glgpu_cg_reset_direction: dir.fill(0)                           (cg.py:264)
 *   glgpu_cg_gradient:        dF/dpsi, dF/dA (cg.h:15-301) and, if
 *                             compute_beta, Polak-Ribiere+ beta   (cg.py:422-449)
 *   glgpu_cg_coefficients:    dir = beta*dir - g, then the 5 (kappa=inf) or 17
 *                             line-search coefficients          (cg.h:314-731, cg.py:184-224,325-375)
 *   glgpu_cg_update:          psi += a_psi dir_psi, A += a_A dir_A, then the
 *                             free energy                       (cg.py:298-311,515-537) */
int glgpu_cg_reset_direction(glgpu_handle* h);
int glgpu_cg_gradient(glgpu_handle* h, int32_t compute_beta);
int glgpu_cg_coefficients(glgpu_handle* h, double* c);            /* 5 or 17 doubles */
int glgpu_cg_update(glgpu_handle* h, double alpha_psi, double alpha_A, double* energy);

/* --- kernel-level test hooks used by the reference's tests
 *     (CG._free_energy_jacobian_psi/_A, cg.py:112-181;
 *      CG._free_energy_conjgrad_coef(_psi), cg.py:184-224,325-375) */
int glgpu_jacobian(glgpu_handle* h, void* g_psi, void* g_A);       /* g_A may be NULL */
int glgpu_conjgrad_coef(glgpu_handle* h, const void* dpsi, const void* dab, double* c);  /* dab NULL: 5 coefficients */

/* --- FP64 vector sum in one launch (the reduction behind every energy/coefficient
 *     sum), exposed as the reference's reduction test hook Reduction.gsum/gsum_v
 *     (svirl/parallel/reduction.py:40-173,179-198).  x: n vectors of nv doubles
 *     (nv = 1, 5 or 17), out: nv sums. */
int glgpu_reduce_sum(glgpu_handle* h, const double* x, int64_t n, int32_t nv, double* out);

/* --- batches: several instances (any sizes and parameters; one dtype, one
 *     device) advanced by one device-side TD loop.  No counterpart in the
 *     reference, which runs one solver per process (svirl/config.py); each
 *     instance follows TD._solve (svirl/solvers/td.py:342-377) with its own
 *     Jacobi stop rule, exactly as if it ran alone.  The batch references the
 *     handles (it does not own them); their state is read and written in place. */
typedef struct glgpu_batch glgpu_batch;
int glgpu_batch_create(glgpu_handle* const* handles, int32_t n, glgpu_batch** out);
int glgpu_batch_destroy(glgpu_batch* b);
const char* glgpu_batch_last_error(const glgpu_batch* b);
int glgpu_batch_td(glgpu_batch* b, double dt, int32_t Nt, int32_t eqn, glgpu_td_stats* stats, double* elapsed_ms);
int glgpu_batch_set_use_graphs(glgpu_batch* b, int32_t enable);
int glgpu_batch_set_loop_guard(glgpu_batch* b, int32_t launches);  /* as glgpu_set_loop_guard */
/* Free-energy minimisation of every instance of the batch with the step
 * length, beta and stop test decided on the device (one graph launch for the
 * whole run).  No counterpart in the reference; each instance follows the
 * Polak-Ribiere+ CG of svirl/solvers/cg.py:238-318 (kappa = inf) and
 * cg.py:452-544 (finite kappa) from a zero direction, with alpha chosen as the
 * smallest non-negative stationary point of the quartic (kappa = inf) or by a
 * damped Newton descent of the (alpha_psi, alpha_A) polynomial from (0, 0)
 * (finite kappa) instead of numpy roots / scipy BFGS on the host.  Stops per
 * instance after n_iter updates, when |E_k/E_{k-1} - 1| < rtol (cg.py:315-318),
 * or when |grad F| <= gtol |grad F of the first iteration| (gtol = 0: off;
 * with GLGPU_CG_GTOL_ABS: |grad F| <= gtol, tested before the first update too).
 * Per-instance outputs (each may be NULL): iterations done, final energy,
 * final |grad F| relative to the first, status (1 gradient stop, 2 energy stop,
 * 3 n_iter reached, 4 energy target reached, 5 energy window (see
 * glgpu_batch_set_cg_window), -1 no descent step; then
 * GLGPU_E_NOROOT is returned).
 * flags: GLGPU_CG_EXACT_BOUNDARY makes dF/dA the exact derivative of the free
 * energy on the boundary links too; the reference's formula (cg.h:174-300)
 * doubles the H and A terms there, so its gradient does not vanish at the
 * energy minimum and the gradient-norm stop cannot be met at finite kappa. */
/* Energy targets for the next glgpu_batch_cg calls: instance q also stops (status
 * 4) once its energy E <= targets[q] + rel_tol |targets[q]| (a NaN target: no
 * such stop; targets = NULL clears them).  Measures the iterations a start needs
 * to reach a known minimum energy. */
int glgpu_batch_set_energy_targets(glgpu_batch* b, const double* targets, double rel_tol);
/* Energy-window stop for the next glgpu_batch_cg calls: every `window` iterations
 * an instance compares its energy with the energy `window` iterations before and
 * stops (status 5) unless it fell by more than rel_tol |E| (window = 0: off).
 * For FP32 batches, whose gradient norm has a rounding floor above tight
 * gradient tolerances: the run ends once the energy has stopped improving. */
int glgpu_batch_set_cg_window(glgpu_batch* b, int32_t window, double rel_tol);
#define GLGPU_CG_EXACT_BOUNDARY 1
#define GLGPU_CG_GTOL_ABS 2
int glgpu_batch_cg(glgpu_batch* b, int32_t n_iter, double rtol, double gtol, int32_t flags, int32_t* iters,
                   double* energies, double* grad_rel, int32_t* status, double* elapsed_ms);

/* --- free energy of a caller-owned state with no allocation by the library.
 *     No counterpart in the reference (its gsum allocates work arrays,
 *     svirl/parallel/reduction.py:165-172).  For callers that must not let a
 *     library call cudaMalloc (their own allocator or a fixed pre-sized arena owns
 *     the device memory).  psi, ab, abei (nullable), mt (nullable) and energy
 *     (one double) are DEVICE pointers on the current device; stream may be NULL.
 *     Asynchronous: *energy is written when the stream reaches the kernel.  The
 *     reduction scratch is a static 256 KB device array in the library (held by
 *     every GPU that loads it until exit), so grids are limited to 8,388,608
 *     nodes (larger ones: GLGPU_E_ARG).  Every call outside stream capture looks
 *     the array up (cudaGetSymbolAddress; a device reset moves it); a call under
 *     capture uses the address of the last call outside capture, so make the
 *     first call on a device before any stream capture.  All calls share the
 *     array: calls that overlap on the GPU race.  The energy uses the scalar
 *     linear coefficient params->epsilon; a spatially varying one (a handle's
 *     glgpu_set_linear_coefficient_field) is not supported by this call. */
int glgpu_free_energy_noalloc(const glgpu_grid* grid, const glgpu_params* params, const void* psi, const void* ab,
                              const void* abei, const uint8_t* mt, double* energy, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GLGPU_H */
