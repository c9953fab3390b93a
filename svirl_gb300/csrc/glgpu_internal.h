// Internal structures of libglgpu: instance descriptors, device-side loop state,
// the handle, and the host-side launch helpers shared by the translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>
#include <vector>

#include "glgpu_common.cuh"
#include "../../include/glgpu.h"

namespace glgpu {

// Temporal blocking of the psi Jacobi loop: one launch of the psi sweep kernel
// does kFuse consecutive sweeps and writes every one of them, so the loop can
// stop after any of them exactly where the one-sweep-per-launch loop stops.
#ifndef GLGPU_FUSE
#define GLGPU_FUSE 3
#endif
constexpr int kFuse = GLGPU_FUSE;
static_assert(kFuse >= 1 && kFuse <= 4, "1 <= GLGPU_FUSE <= 4");
constexpr int kPsiBufs = kFuse + 2;  // right-hand side + input + kFuse outputs
// TD graphs cached per handle / batch: eqn mode (3) x any finite kappa (2) x any
// fixed vortices (2)
constexpr int kTDGraphs = 12;

// Device-resident state of one instance's Jacobi loops (updated by the kernels
// themselves so that a whole TD run needs no host round trip).
struct InstState {
    unsigned long long res;   // A loop: max residual of the current sweep, as IEEE bits
    unsigned long long resp[4];  // psi loop: max residual of each sweep of the current launch
    int nanlv;                // psi loop: bit l set if sweep l of the current launch saw a NaN residual
    unsigned blocks_done;     // CTAs (A) / strips (psi) of this instance finished in the current launch
    int sweep;                // sweeps done in the current Jacobi loop
    int done;                 // current Jacobi loop finished
    int rhs;                  // buffer index (0..kPsiBufs-1) of psi^(0) = right-hand side of the psi loop
    int rhsA;                 // same for the A loop (0..2)
    uint32_t rand_t;          // Langevin time seed (svirl/solvers/td.py:35-37,204,313)
    int nan_seen;             // a NaN residual was seen (the reference counts it as converged)
    int last_sweeps_psi, last_sweeps_A, max_sweeps_psi, max_sweeps_A;
    long long total_sweeps_psi, total_sweeps_A;
    int steps;                // time steps done in the current call
    int commitA;              // FP32 A loop: 1 + the buffer of A^(0) to add to the final offsets (0: none)
};

// Device-resident state of one instance in the batched device CG.
struct CGState {
    double beta_psi, beta_A;
    double c[17];             // line-search coefficients of the current iteration
    double alpha_psi, alpha_A;
    double E, E_prev;         // energy after the last / the previous update
    double g2, g2_0;          // |gradient|^2 now and at the first iteration
    int iter, done, gi, di;   // iterations done, finished, current gradient / direction buffer
    int status;               // 0 ok, 1 gradient-norm stop, 2 energy stop, 3 n_iter, 4 energy target,
                              // 5 energy window (stagnation), -1 no step found
    int pi;                   // buffer (psi[pi], ab[pi]) holding the current state during a CG call
    int ticket;               // CTAs of this instance finished in the running launch
    int it_mark;              // iteration of the last energy-window mark
    double E_mark;            // energy at that mark
};

// Everything a kernel needs to process one instance.  Lives in device memory,
// one entry per instance of a batch (a single GLSolver is a batch of one).
struct Inst {
    Geo g;
    double dt, epsilon, kappa2, rho, H;
    double lang_psi, lang_A;
    double stop_psi, stop_A;
    float fdt, fepsilon, fkappa2, frho, fH, flang_psi, flang_A, pad_f;  // the same, rounded to float
    int lang_psi_on, lang_A_on;  // Langevin coefficient (in the solver's precision) > 1e-32 (td.h:147,451)
    void* psi[kPsiBufs];      // rotating TD buffers, psi[0] holds the state at rest
    void* ab[3];              // rotating TD buffers, ab[0] holds the state at rest
    const void* abei;         // external+irregular vector potential or NULL
    const uint8_t* mt;        // material tiling (cells) or NULL
    const void* eps_sp;       // spatial linear coefficient (nodes) or NULL
    void* U;                  // link factors of the psi loop (Nab complex); during the A loop the
                              // fixed parts of the link updates (k_A_sweep), 2 Nab reals
    uint8_t* code;            // per-node link-weight bits of the psi loop, N bytes
    void* dinv;               // FP64: per-node reciprocal of the psi step's diagonal, N reals (NULL for FP32)
    uint8_t* cbits;           // per-node cell bits (cell_bits) for the batched CG, N bytes (NULL until CG)
    void* vpi;                // irregular vector potential of fixed vortices, Nab, or NULL
    const int32_t* lock;      // phase-lock node list or NULL
    int lock_n, pad_lock;
    InstState* st;
    CGState* cg;              // batched device CG state (NULL until used)
    void* gpsi[2];            // CG gradient buffers (psi part, A part) and directions
    void* gA[2];
    void* dpsi[2];
    void* dA[2];
    int tile0, ntiles;        // this instance's range in the tile table
    int natiles;              // its A-sweep tiles (ATile)
    int nitems;               // number of warp-strip items of this instance
    int solveA;               // finite kappa
    int cg_exact;             // batched device CG: exact dF/dA on boundary links
    double cg_target;         // batched device CG: stop once E <= cg_target + cg_target_tol |cg_target| (NaN: off)
    double cg_target_tol;
};

// Global state of one batched Jacobi/time loop.
struct LoopState {
    int active;               // instances whose current Jacobi loop is not done
    unsigned blocks_done;     // CTAs finished in the current launch
    int launches;             // sweeps launched in the current Jacobi loop
    int cont;                 // last decision of the Jacobi while loop
    int step, Nt;             // time loop position / length
    int err;                  // error bits (kErr*)
    int ninst;
    long long total_launches;  // sweep kernel launches (psi and A) in the current call
    int guard;                // launches after which a Jacobi loop is stopped with kErrLoopGuard
};

constexpr int kErrLoopGuard = 1;
constexpr int kErrCopyWait = 2;  // a wait for a bulk copy into shared memory ran out (psi sweep)

// A tile = 256 consecutive nodes of one instance.
struct Tile {
    int inst, n0;
};

// A tile of the A sweep: kATX x kATY nodes of one instance from node (i0, j0)
// (a CTA of 256 threads covers 256 / kATX rows of the tile per pass).  64 x 32:
// 0.084 ms per sweep at 2049^2 and kappa = 4; 32 x 32, 64 x 16 and 128 x 8 tiles
// 0.090-0.091 ms, 32 x 64 and 128 x 16 0.084-0.085.
#ifndef GLGPU_ATX
#define GLGPU_ATX 64
#endif
#ifndef GLGPU_ATY
#define GLGPU_ATY 32
#endif
constexpr int kATX = GLGPU_ATX, kATY = GLGPU_ATY;
static_assert(256 % kATX == 0 && kATY % (256 / kATX) == 0, "A tile: whole rows per pass, whole passes per tile");
struct ATile {
    int inst, i0, j0, pad;
};
inline int atiles_of(int Nx, int Ny) { return ((Nx + kATX - 1) / kATX) * ((Ny + kATY - 1) / kATY); }

// Work item of the warp-strip psi sweep: kStripCols output columns (x0..) by
// `rows` rows (j0..) of one instance, processed by one warp whose 32 lanes also
// cover kFuse halo columns on each side.  The sweep kernel is compiled for the
// strip heights of kStripRowsSet; a handle or batch uses the one that
// choose_strip_rows (td.cu) picks for its item count.
#ifdef GLGPU_STRIP_ROWS
constexpr int kStripRowsSet[] = {GLGPU_STRIP_ROWS};
#else
constexpr int kStripRowsSet[] = {8, 12, 17};
#endif
constexpr int kNumStripRows = (int)(sizeof(kStripRowsSet) / sizeof(kStripRowsSet[0]));
constexpr int kStripCols = 32 - 2 * kFuse;
inline int strip_items(int Nx, int Ny, int rows) {
    return ((Nx + kStripCols - 1) / kStripCols) * ((Ny + rows - 1) / rows);
}
// The FP32 sweep runs kPsiGroup adjacent strips of one row band per CTA (they
// share one ring of rows in shared memory), so the item table lists each band's
// strips in groups of kPsiGroup, the last group of a band padded with empty
// items (inst = -1).  strip_table_len: entries of one instance's table.
constexpr int kPsiGroup = 4;
inline int strip_table_len(int Nx, int Ny, int rows) {
    const int nstrips = (Nx + kStripCols - 1) / kStripCols;
    return (nstrips + kPsiGroup - 1) / kPsiGroup * kPsiGroup * ((Ny + rows - 1) / rows);
}
struct Item {
    int inst, x0, j0, pad;  // inst = -1: an empty item (group padding)
};

}  // namespace glgpu

// The opaque handle behind glgpu_handle*: one instance with its buffers.
struct glgpu_handle {
    int dtype;                   // 4 or 8
    glgpu::Geo g;
    glgpu_params p;
    cudaStream_t stream = nullptr;
    int device = 0;
    // device buffers
    void* psi[glgpu::kPsiBufs] = {};
    void* ab[3] = {nullptr, nullptr, nullptr};
    void* abei = nullptr;
    uint8_t* mt = nullptr;
    void* eps_sp = nullptr;
    void* U = nullptr;
    uint8_t* code = nullptr;
    void* dinv = nullptr;
    glgpu::InstState* st = nullptr;
    glgpu::Inst* inst = nullptr;        // device copy of the descriptor
    glgpu::Inst inst_h;                 // host copy of the descriptor
    glgpu::Tile* tiles = nullptr;
    glgpu::ATile* atiles = nullptr;     // A-sweep tiles
    int natiles = 0;
    glgpu::Item* items = nullptr;
    int nitems = 0;
    int strip_rows = 0;                 // strip height of the psi sweep items
    int psi_grid = 0;                   // CTAs of the persistent psi sweep
    glgpu::LoopState* loop = nullptr;
    int ntiles = 0;
    // reductions / outputs
    double* partials = nullptr;         // nblocks * 17 doubles
    unsigned* counter = nullptr;        // ticket counter for grid_sum_finish
    double* dscal = nullptr;            // device scalars: [0..16] coefficients, [20] energy, [24..27] beta sums, [28] beta_psi, [29] beta_A
    void* out = nullptr;                // staging buffer for observables (Nab reals, Nc reals)
    void* vort = nullptr;               // vortex candidates
    int* vort_n = nullptr;
    int vort_cap = 0;
    // CG buffers (allocated on first use)
    void* g_psi[2] = {nullptr, nullptr};
    void* g_A[2] = {nullptr, nullptr};
    void* dir_psi[2] = {nullptr, nullptr};
    void* dir_A[2] = {nullptr, nullptr};
    int cg_g = 0, cg_dir = 0;           // current index of g / dir
    glgpu::CGState* cgst = nullptr;     // batched device CG state
    void* vpi = nullptr;                // irregular vector potential (fixed vortices), Nab, or NULL (the TD step's copy)
    int32_t* lock = nullptr;            // phase-lock node list (fixed vortices) or NULL
    int lock_n = 0;
    uint8_t* cbits = nullptr;           // batched CG: cell bits per node, written at the start of a call
    // TD graphs, one per (equation mode, kappa finite)
    cudaGraphExec_t td_exec[glgpu::kTDGraphs] = {};
    glgpu::InstState* st_gather = nullptr;  // device copy target of the loop state
    bool td_graph_failed = false;
    bool use_graphs = true;
    int loop_guard = 0;                 // Jacobi loop guard in sweep launches (0: kLoopGuard)
    int psi_select = 0;                 // psi sweep kernel (psi_kind)
    int psi_scheme = 0;                 // psi time stepping: 0 backward Euler, 1 Crank-Nicolson, 2 as written
    std::string last_error;
    void* flush = nullptr;              // L2 flush buffer for kernel timing
    // host pinned staging for small results
    double* hscal = nullptr;
    void* pin = nullptr;                // PinStage (pinned host memory)
};

// A batch: several handles (instances of any sizes and parameters, one dtype,
// one device) advanced together.  Their descriptors, item and tile tables are
// concatenated, so one sweep launch covers every instance and each instance
// keeps its own Jacobi stop rule.
// Pinned host staging of a handle's per-call copies (descriptor up, loop state and
// statistics down).
struct PinStage {
    glgpu::Inst inst;
    glgpu::InstState st;
    glgpu::LoopState loop;
};

struct glgpu_batch {
    int dtype = 4, device = 0, ninst = 0;
    std::vector<glgpu_handle*> hs;
    cudaStream_t stream = nullptr;
    glgpu::Inst* insts = nullptr;
    glgpu::Tile* tiles = nullptr;
    glgpu::ATile* atiles = nullptr;     // A-sweep tiles
    int natiles = 0;
    glgpu::Item* items = nullptr;
    glgpu::LoopState* loop = nullptr;
    glgpu::InstState* gather = nullptr;
    std::vector<glgpu::InstState> gather_h;
    glgpu::InstState* gather_pin = nullptr;  // pinned host copies of the per-call transfers
    glgpu::LoopState* loop_pin = nullptr;
    glgpu::Inst* insts_pin = nullptr;
    int ntiles = 0, nitems = 0, psi_grid = 0, strip_rows = 0;
    std::vector<int> inst_items;         // psi sweep items of each instance (at strip_rows)
    cudaGraphExec_t td_exec[glgpu::kTDGraphs] = {};
    bool td_graph_failed = false, use_graphs = true;
    int loop_guard = 0;                  // Jacobi loop guard in sweep launches (0: kLoopGuard)
    // batched device CG (allocated on first use)
    void* cg_tiles = nullptr;            // CG tile table (larger tiles than the TD one)
    int cg_ntiles = 0;
    double* cg_partials = nullptr;       // cg_ntiles * 17 doubles
    void* cg_loop = nullptr;             // CGLoop
    cudaGraphExec_t cg_exec = nullptr;
    bool cg_graph_failed = false;
    std::vector<double> cg_targets;      // per-instance energy targets (empty: none)
    double cg_target_tol = 0.0;
    int cg_window = 0;                   // energy-window stop: iterations (0: off) and relative decrease
    double cg_window_tol = 0.0;
    std::string last_error;
};

namespace glgpu {

int batch_error(glgpu_batch* b, int code, const std::string& msg);
int batch_td(glgpu_batch* b, double dt, int Nt, int eqn, glgpu_td_stats* stats, double* elapsed_ms);
int set_error(glgpu_handle* h, int code, const std::string& msg);
int cuda_check(glgpu_handle* h, cudaError_t e, const char* what);
void upload_inst(glgpu_handle* h);
size_t real_size(const glgpu_handle* h);

// td.cu
int td_run(glgpu_handle* h, double dt, int Nt, int eqn, glgpu_td_stats* stats, double* elapsed_ms);
int time_sweeps(glgpu_handle* h, int which, int nrep, double* avg_ms);
int choose_strip_rows(int dtype, const Geo* const* geos, int n);
// psi sweep kernel of a dtype and a selection (0: register strip, the default;
// 1: FP32 bulk-copy ring): 8 = FP64 register strip, 4 = FP32 register strip,
// 5 = FP32 bulk-copy ring
inline int psi_kind(int dtype, int select) { return dtype == 8 ? 8 : (select == 1 ? 5 : 4); }
int psi_sweep_grid(int kind, int rows, int nitems);
std::vector<Item> make_items(const Geo& g, int inst, int rows);
// obs.cu
int obs_free_energy(glgpu_handle* h, double* out);
int obs_magnetic_field(glgpu_handle* h, void* host_out);
int obs_current_density(glgpu_handle* h, void* host_out);
int obs_supercurrent_density(glgpu_handle* h, void* host_out);
int obs_vortex_candidates(glgpu_handle* h, int cap, int* n_out, int32_t* cells, void* corners);
int reduce_sum(glgpu_handle* h, const double* x, long long n, int nv, double* out);
int free_energy_noalloc(const glgpu_grid* grid, const glgpu_params* p, const void* psi, const void* ab,
                        const void* abei, const uint8_t* mt, double* energy, cudaStream_t stream);
// cg.cu
int cg_ensure(glgpu_handle* h);
int cg_reset_direction(glgpu_handle* h);
int cg_gradient(glgpu_handle* h, int compute_beta);
int cg_coefficients(glgpu_handle* h, double* c_out);
int cg_update(glgpu_handle* h, double alpha_psi, double alpha_A, double* energy_out);
int cg_read_gradient(glgpu_handle* h, void* gpsi_host, void* gA_host);
int cg_coef_for(glgpu_handle* h, const void* dpsi_host, const void* dab_host, double* c_out);
// cgb.cu
int batch_set_energy_targets(glgpu_batch* b, const double* targets, double rel_tol);
int batch_set_cg_window(glgpu_batch* b, int window, double rel_tol);
int batch_cg(glgpu_batch* b, int n_iter, double rtol, double gtol, int flags, int32_t* iters, double* energies, double* grad_rel,
             int32_t* status, double* elapsed_ms);
// td.cu graph helpers
cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, int ndeps, void* fn, dim3 grid,
                       dim3 block, void** args, unsigned smem_bytes = 0);
cudaError_t add_while(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, int ndeps,
                      cudaGraphConditionalHandle h, cudaGraph_t* body);

inline int blocks_for(long long n) { return (int)((n + kThreads - 1) / kThreads); }

}  // namespace glgpu
