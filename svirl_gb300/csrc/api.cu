// C ABI of libglgpu: handle lifetime, state and parameter transfer, and the
// extern "C" wrappers of the TD / CG / observable entry points.
#include <cmath>
#include <algorithm>
#include <cstring>
#include <string>

#include "glgpu_internal.h"

using namespace glgpu;

static thread_local std::string g_create_error;

namespace glgpu {

int set_error(glgpu_handle* h, int code, const std::string& msg) {
    if (h) h->last_error = msg;
    else g_create_error = msg;
    return code;
}

int cuda_check(glgpu_handle* h, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return GLGPU_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_error(h, GLGPU_E_OOM, m);
    return set_error(h, GLGPU_E_CUDA, m);
}

size_t real_size(const glgpu_handle* h) { return (size_t)h->dtype; }

int batch_error(glgpu_batch* b, int code, const std::string& msg) {
    if (b) b->last_error = msg;
    return code;
}

static bool finite_kappa(const glgpu_params& p) { return p.kappa > 0.0 && !std::isinf(p.kappa); }

void upload_inst(glgpu_handle* h) {
    Inst I;
    memset(&I, 0, sizeof(I));
    I.g = h->g;
    I.dt = 0.0;
    I.epsilon = h->p.epsilon;
    I.kappa2 = finite_kappa(h->p) ? h->p.kappa * h->p.kappa : -1.0;
    I.rho = 1.0 / h->p.sigma;
    I.H = h->p.H;
    I.lang_psi = h->p.langevin_psi;
    I.lang_A = h->p.langevin_A;
    const double lo = h->dtype == 4 ? 1e-6 : 1e-12;  // svirl/solvers/td.py:52-66
    I.stop_psi = h->p.stop_psi < lo ? lo : h->p.stop_psi;
    I.stop_A = h->p.stop_A < lo ? lo : h->p.stop_A;
    if (h->dtype == 4) {
        I.stop_psi = (double)(float)I.stop_psi;
        I.stop_A = (double)(float)I.stop_A;
    }
    for (int q = 0; q < kPsiBufs; ++q) I.psi[q] = h->psi[q];
    for (int q = 0; q < 3; ++q) I.ab[q] = h->ab[q];
    I.abei = h->abei;
    I.mt = h->mt;
    I.eps_sp = h->eps_sp;
    I.U = h->U;
    I.code = h->code;
    I.dinv = h->dinv;
    I.st = h->st;
    I.cg = h->cgst;
    I.cbits = h->cbits;
    I.vpi = h->vpi;
    I.lock = h->lock;
    I.lock_n = h->lock_n;
    for (int q = 0; q < 2; ++q) {
        I.gpsi[q] = h->g_psi[q];
        I.gA[q] = h->g_A[q];
        I.dpsi[q] = h->dir_psi[q];
        I.dA[q] = h->dir_A[q];
    }
    I.tile0 = 0;
    I.ntiles = h->ntiles;
    I.natiles = h->natiles;
    I.nitems = strip_items(h->g.Nx, h->g.Ny, h->strip_rows);  // strips (the table also has empty items)
    I.solveA = finite_kappa(h->p) ? 1 : 0;
    I.fepsilon = (float)I.epsilon;
    I.fkappa2 = (float)I.kappa2;
    I.frho = (float)I.rho;
    I.fH = (float)I.H;
    I.flang_psi = (float)I.lang_psi;
    I.flang_A = (float)I.lang_A;
    I.lang_psi_on = (h->dtype == 4 ? (double)I.flang_psi : I.lang_psi) > 1.0e-32 ? 1 : 0;
    I.lang_A_on = (h->dtype == 4 ? (double)I.flang_A : I.lang_A) > 1.0e-32 ? 1 : 0;
    I.dt = h->inst_h.dt;
    I.fdt = (float)I.dt;
    h->inst_h = I;
    cudaMemcpyAsync(h->inst, &h->inst_h, sizeof(Inst), cudaMemcpyHostToDevice, h->stream);
}

}  // namespace glgpu

static int check_handle(const glgpu_handle* h) { return h ? GLGPU_OK : GLGPU_E_ARG; }

static void free_all(glgpu_handle* h) {
    for (int q = 0; q < kPsiBufs; ++q)
        if (h->psi[q]) cudaFree(h->psi[q]);
    for (int q = 0; q < 3; ++q)
        if (h->ab[q]) cudaFree(h->ab[q]);
    for (int q = 0; q < kTDGraphs; ++q)
        if (h->td_exec[q]) cudaGraphExecDestroy(h->td_exec[q]);
    if (h->st_gather) cudaFree(h->st_gather);
    if (h->cgst) cudaFree(h->cgst);
    if (h->cbits) cudaFree(h->cbits);
    if (h->vpi) cudaFree(h->vpi);
    if (h->lock) cudaFree(h->lock);
    for (int q = 0; q < 2; ++q) {
        if (h->g_psi[q]) cudaFree(h->g_psi[q]);
        if (h->g_A[q]) cudaFree(h->g_A[q]);
        if (h->dir_psi[q]) cudaFree(h->dir_psi[q]);
        if (h->dir_A[q]) cudaFree(h->dir_A[q]);
    }
    void* ptrs[] = {h->abei, h->mt, h->eps_sp, h->U, h->code, h->dinv, h->st, h->inst, h->tiles, h->atiles, h->items, h->loop, h->partials, h->counter,
                    h->dscal, h->out, h->vort, h->vort_n, h->flush};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->hscal) cudaFreeHost(h->hscal);
    if (h->pin) cudaFreeHost(h->pin);
    if (h->stream) cudaStreamDestroy(h->stream);
}

extern "C" {

int glgpu_version(void) { return 10000; }

int glgpu_psi_sweeps_per_launch(void) { return kFuse; }

int glgpu_psi_strip_rows(const glgpu_handle* h) { return h ? h->strip_rows : 0; }

const char* glgpu_last_error(const glgpu_handle* h) { return h ? h->last_error.c_str() : g_create_error.c_str(); }

int glgpu_create(const glgpu_grid* grid, int32_t device, glgpu_handle** out) {
    if (!grid || !out) return set_error(nullptr, GLGPU_E_ARG, "glgpu_create: NULL argument");
    *out = nullptr;
    if (grid->Nx < 4 || grid->Ny < 4) return set_error(nullptr, GLGPU_E_ARG, "glgpu_create: Nx and Ny must be >= 4");
    if (grid->dtype != 4 && grid->dtype != 8) return set_error(nullptr, GLGPU_E_ARG, "glgpu_create: dtype must be 4 or 8");
    if (!(grid->dx > 0.0) || !(grid->dy > 0.0)) return set_error(nullptr, GLGPU_E_ARG, "glgpu_create: dx, dy must be > 0");
    if ((long long)grid->Nx * grid->Ny > (1LL << 30)) return set_error(nullptr, GLGPU_E_ARG, "glgpu_create: grid too large");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return set_error(nullptr, GLGPU_E_CUDA, std::string("glgpu_create: cudaSetDevice: ") + cudaGetErrorString(e));
    glgpu_handle* h = new glgpu_handle();
    h->device = device;
    h->dtype = grid->dtype;
    h->g = make_geo(grid->Nx, grid->Ny, grid->dx, grid->dy);
    memset(&h->p, 0, sizeof(h->p));
    h->p.kappa = INFINITY;
    h->p.sigma = 1.0;
    h->p.epsilon = 1.0;
    h->p.stop_psi = 1e-6;
    h->p.stop_A = 1e-6;
    h->p.rand_t = 1;
    const size_t rs = (size_t)h->dtype;
    const size_t npsi = (size_t)h->g.N * 2 * rs, nab = (size_t)h->g.Nab * rs;
    h->ntiles = blocks_for(h->g.N);
    const int nblk = blocks_for(h->g.N);
    bool ok = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess;
    // 64 bytes of slack after psi and the code table: the FP32 sweep copies whole
    // 16-byte units, which can reach up to 15 bytes past a row's last node
    for (int q = 0; q < kPsiBufs && ok; ++q) ok = cudaMalloc(&h->psi[q], npsi + 64) == cudaSuccess;
    for (int q = 0; q < 3 && ok; ++q) ok = cudaMalloc(&h->ab[q], nab) == cudaSuccess;
    // link factors: Nab complex for the CG, one (x link, y link) pair per node for the TD step
    ok = ok && cudaMalloc(&h->U, std::max((size_t)h->g.Nab * 2, (size_t)h->g.N * 4) * rs) == cudaSuccess;
    ok = ok && cudaMalloc(&h->code, (size_t)h->g.N + 64) == cudaSuccess;
    if (h->dtype == 8) ok = ok && cudaMalloc(&h->dinv, (size_t)h->g.N * rs) == cudaSuccess;
    ok = ok && cudaMalloc(&h->st, sizeof(InstState)) == cudaSuccess;
    ok = ok && cudaMalloc(&h->st_gather, sizeof(InstState)) == cudaSuccess;
    ok = ok && cudaMalloc(&h->inst, sizeof(Inst)) == cudaSuccess;
    ok = ok && cudaMalloc(&h->tiles, sizeof(Tile) * (size_t)h->ntiles) == cudaSuccess;
    h->natiles = atiles_of(h->g.Nx, h->g.Ny);
    ok = ok && cudaMalloc(&h->atiles, sizeof(ATile) * (size_t)h->natiles) == cudaSuccess;
    {
        const Geo* gp = &h->g;
        h->strip_rows = choose_strip_rows(h->dtype, &gp, 1);
    }
    h->nitems = strip_table_len(h->g.Nx, h->g.Ny, h->strip_rows);
    ok = ok && cudaMalloc(&h->items, sizeof(Item) * (size_t)h->nitems) == cudaSuccess;
    ok = ok && cudaMalloc(&h->loop, sizeof(LoopState)) == cudaSuccess;
    ok = ok && cudaMalloc(&h->partials, sizeof(double) * 17 * (size_t)nblk) == cudaSuccess;
    ok = ok && cudaMalloc(&h->counter, sizeof(unsigned) * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&h->dscal, sizeof(double) * 32) == cudaSuccess;
    ok = ok && cudaMalloc(&h->out, nab > (size_t)h->g.Nxc * h->g.Nyc * rs ? nab : (size_t)h->g.Nxc * h->g.Nyc * rs) == cudaSuccess;
    ok = ok && cudaMalloc(&h->vort_n, sizeof(int)) == cudaSuccess;
    ok = ok && cudaMallocHost(&h->hscal, sizeof(double) * 32) == cudaSuccess;
    ok = ok && cudaMallocHost(&h->pin, sizeof(PinStage)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_all(h);
        delete h;
        return set_error(nullptr, GLGPU_E_OOM, "glgpu_create: device allocation failed");
    }
    std::vector<Tile> tiles(h->ntiles);
    for (int k = 0; k < h->ntiles; ++k) tiles[k] = Tile{0, k * kThreads};
    const std::vector<Item> items = make_items(h->g, 0, h->strip_rows);
    h->psi_grid = psi_sweep_grid(psi_kind(h->dtype, h->psi_select), h->strip_rows, h->nitems);
    InstState st;
    memset(&st, 0, sizeof(st));
    st.rand_t = h->p.rand_t;
    std::vector<ATile> atiles;
    for (int j0 = 0; j0 < h->g.Ny; j0 += kATY)
        for (int i0 = 0; i0 < h->g.Nx; i0 += kATX) atiles.push_back(ATile{0, i0, j0, 0});
    e = cudaMemcpyAsync(h->tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->atiles, atiles.data(), sizeof(ATile) * atiles.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->items, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->st, &st, sizeof(st), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->counter, 0, sizeof(unsigned) * 4, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->dscal, 0, sizeof(double) * 32, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->loop, 0, sizeof(LoopState), h->stream);
    for (int q = 0; q < kPsiBufs && e == cudaSuccess; ++q) e = cudaMemsetAsync(h->psi[q], 0, npsi, h->stream);
    for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = cudaMemsetAsync(h->ab[q], 0, nab, h->stream);
    if (e == cudaSuccess && h->dinv) e = cudaMemsetAsync(h->dinv, 0, (size_t)h->g.N * rs, h->stream);
    if (e == cudaSuccess) {
        upload_inst(h);
        e = cudaStreamSynchronize(h->stream);
    }
    if (e != cudaSuccess) {
        std::string m = std::string("glgpu_create: ") + cudaGetErrorString(e);
        free_all(h);
        delete h;
        return set_error(nullptr, GLGPU_E_CUDA, m);
    }
    *out = h;
    return GLGPU_OK;
}

int glgpu_destroy(glgpu_handle* h) {
    if (!h) return GLGPU_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return GLGPU_OK;
}

int glgpu_set_params(glgpu_handle* h, const glgpu_params* p) {
    if (check_handle(h) || !p) return set_error(h, GLGPU_E_ARG, "set_params: NULL argument");
    if (!(p->sigma > 0.0)) return set_error(h, GLGPU_E_ARG, "set_params: normal_conductivity must be > 0");
    if (!(p->stop_psi > 0.0) || !(p->stop_A > 0.0)) return set_error(h, GLGPU_E_ARG, "set_params: stop criteria must be > 0");
    const bool was_finite = finite_kappa(h->p), now_finite = finite_kappa(*p);
    h->p = *p;
    (void)was_finite;  // the TD graphs are kept per (equation mode, kappa finite)
    (void)now_finite;
    upload_inst(h);
    cudaError_t e = cudaMemcpyAsync(&h->st->rand_t, &h->p.rand_t, sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return cuda_check(h, e, "set_params");
}

int glgpu_get_params(const glgpu_handle* h, glgpu_params* p) {
    if (!h || !p) return GLGPU_E_ARG;
    *p = h->p;
    return GLGPU_OK;
}

static int h2d(glgpu_handle* h, void* dst, const void* src, size_t bytes, const char* what) {
    if (!src) return set_error(h, GLGPU_E_ARG, std::string(what) + ": NULL buffer");
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, h->stream);  // host or device source
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return cuda_check(h, e, what);
}

static int d2h(glgpu_handle* h, void* dst, const void* src, size_t bytes, const char* what) {
    if (!dst) return set_error(h, GLGPU_E_ARG, std::string(what) + ": NULL buffer");
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, h->stream);  // host or device target
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return cuda_check(h, e, what);
}

int glgpu_set_order_parameter(glgpu_handle* h, const void* psi) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return h2d(h, h->psi[0], psi, (size_t)h->g.N * 2 * real_size(h), "set_order_parameter");
}

int glgpu_get_order_parameter(glgpu_handle* h, void* psi) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return d2h(h, psi, h->psi[0], (size_t)h->g.N * 2 * real_size(h), "get_order_parameter");
}

int glgpu_set_vector_potential(glgpu_handle* h, const void* ab) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return h2d(h, h->ab[0], ab, (size_t)h->g.Nab * real_size(h), "set_vector_potential");
}

int glgpu_get_vector_potential(glgpu_handle* h, void* ab) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return d2h(h, ab, h->ab[0], (size_t)h->g.Nab * real_size(h), "get_vector_potential");
}

static int set_optional(glgpu_handle* h, void** slot, const void* src, size_t bytes, const char* what) {
    if (!src) {
        if (*slot) {
            cudaStreamSynchronize(h->stream);
            cudaFree(*slot);
            *slot = nullptr;
        }
        upload_inst(h);
        return cuda_check(h, cudaStreamSynchronize(h->stream), what);
    }
    if (!*slot && cudaMalloc(slot, bytes) != cudaSuccess) {
        *slot = nullptr;
        return set_error(h, GLGPU_E_OOM, std::string(what) + ": out of device memory");
    }
    upload_inst(h);
    return h2d(h, *slot, src, bytes, what);
}

int glgpu_set_external_vector_potential(glgpu_handle* h, const void* abei) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return set_optional(h, &h->abei, abei, (size_t)h->g.Nab * real_size(h), "set_external_vector_potential");
}

int glgpu_set_material_tiling(glgpu_handle* h, const uint8_t* mt) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return set_optional(h, (void**)&h->mt, mt, (size_t)h->g.Nxc * h->g.Nyc, "set_material_tiling");
}

int glgpu_set_linear_coefficient_field(glgpu_handle* h, const void* eps) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return set_optional(h, &h->eps_sp, eps, (size_t)h->g.N * real_size(h), "set_linear_coefficient_field");
}

int glgpu_set_use_graphs(glgpu_handle* h, int32_t enable) {
    if (check_handle(h)) return GLGPU_E_ARG;
    h->use_graphs = enable != 0;
    return GLGPU_OK;
}

int glgpu_set_loop_guard(glgpu_handle* h, int32_t launches) {
    if (check_handle(h)) return GLGPU_E_ARG;
    if (launches < 0) return set_error(h, GLGPU_E_ARG, "set_loop_guard: launches must be >= 0");
    h->loop_guard = launches;
    return GLGPU_OK;
}

static void drop_td_graphs(glgpu_handle* h) {
    for (int q = 0; q < kTDGraphs; ++q)
        if (h->td_exec[q]) {
            cudaGraphExecDestroy(h->td_exec[q]);
            h->td_exec[q] = nullptr;
        }
}

int glgpu_set_psi_scheme(glgpu_handle* h, int32_t scheme) {
    if (check_handle(h)) return GLGPU_E_ARG;
    if (scheme < 0 || scheme > 2) return set_error(h, GLGPU_E_ARG, "set_psi_scheme: scheme is 0, 1 or 2");
    cudaSetDevice(h->device);
    if (scheme == h->psi_scheme) return GLGPU_OK;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "set_psi_scheme");
    h->psi_scheme = scheme;
    drop_td_graphs(h);  // the TD graphs hold the sweep kernel
    return GLGPU_OK;
}

int glgpu_set_psi_sweep_kernel(glgpu_handle* h, int32_t select) {
    if (check_handle(h)) return GLGPU_E_ARG;
    if (select < 0 || select > 1) return set_error(h, GLGPU_E_ARG, "set_psi_sweep_kernel: select is 0 or 1");
    cudaSetDevice(h->device);
    if (select == h->psi_select) return GLGPU_OK;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "set_psi_sweep_kernel");
    h->psi_select = select;
    h->psi_grid = psi_sweep_grid(psi_kind(h->dtype, h->psi_select), h->strip_rows, h->nitems);
    drop_td_graphs(h);  // the TD graphs hold the kernel and its grid
    return GLGPU_OK;
}

int glgpu_set_psi_strip_rows(glgpu_handle* h, int32_t rows) {
    if (check_handle(h)) return GLGPU_E_ARG;
    cudaSetDevice(h->device);
    if (rows == 0) {
        const Geo* gp = &h->g;
        rows = choose_strip_rows(h->dtype, &gp, 1);
    }
    bool known = false;
    for (int v = 0; v < kNumStripRows; ++v) known = known || kStripRowsSet[v] == rows;
    if (!known) return set_error(h, GLGPU_E_ARG, "set_psi_strip_rows: strip height not compiled in");
    if (rows == h->strip_rows) return GLGPU_OK;
    const std::vector<Item> items = make_items(h->g, 0, rows);
    Item* buf = nullptr;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = cudaMalloc(&buf, sizeof(Item) * items.size());
    if (e == cudaSuccess) e = cudaMemcpy(buf, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (buf) cudaFree(buf);
        return cuda_check(h, e, "set_psi_strip_rows");
    }
    cudaFree(h->items);
    h->items = buf;
    h->strip_rows = rows;
    h->nitems = (int)items.size();
    h->psi_grid = psi_sweep_grid(psi_kind(h->dtype, h->psi_select), rows, h->nitems);
    drop_td_graphs(h);  // the TD graphs hold the old kernel, grid and table
    upload_inst(h);
    return cuda_check(h, cudaStreamSynchronize(h->stream), "set_psi_strip_rows");
}

int glgpu_set_irregular_vector_potential(glgpu_handle* h, const void* vpi, int32_t td_copy_only) {
    if (check_handle(h)) return GLGPU_E_ARG;
    cudaSetDevice(h->device);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "set_irregular_vector_potential");
    const size_t bytes = (size_t)h->g.Nab * real_size(h);
    if (!vpi) {
        if (h->vpi) cudaFree(h->vpi);
        h->vpi = nullptr;
    } else if (td_copy_only) {
        if (!h->vpi) return set_error(h, GLGPU_E_ARG, "set_irregular_vector_potential: no irregular potential set");
        e = cudaMemcpy(h->vpi, vpi, bytes, cudaMemcpyDefault);
        if (e != cudaSuccess) return cuda_check(h, e, "set_irregular_vector_potential");
    } else {
        if (!h->vpi && cudaMalloc(&h->vpi, bytes) != cudaSuccess)
            return set_error(h, GLGPU_E_OOM, "set_irregular_vector_potential: out of device memory");
        e = cudaMemcpy(h->vpi, vpi, bytes, cudaMemcpyDefault);
        if (e != cudaSuccess) return cuda_check(h, e, "set_irregular_vector_potential");
    }
    drop_td_graphs(h);
    upload_inst(h);
    return cuda_check(h, cudaStreamSynchronize(h->stream), "set_irregular_vector_potential");
}

int glgpu_get_irregular_vector_potential(glgpu_handle* h, void* out) {
    if (check_handle(h) || !out) return GLGPU_E_ARG;
    cudaSetDevice(h->device);
    const size_t bytes = (size_t)h->g.Nab * real_size(h);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) {
        if (h->vpi) {
            e = cudaMemcpy(out, h->vpi, bytes, cudaMemcpyDefault);
        } else {
            const std::vector<unsigned char> zeros(bytes, 0);
            e = cudaMemcpy(out, zeros.data(), bytes, cudaMemcpyDefault);
        }
    }
    return cuda_check(h, e, "get_irregular_vector_potential");
}

int glgpu_set_phase_lock(glgpu_handle* h, const int32_t* nodes, int32_t count) {
    if (check_handle(h) || count < 0 || (count > 0 && !nodes)) return GLGPU_E_ARG;
    for (int32_t k = 0; k < count; ++k)
        if (nodes[k] < 0 || nodes[k] >= h->g.N) return set_error(h, GLGPU_E_ARG, "set_phase_lock: node index out of range");
    if (count > h->g.N) return set_error(h, GLGPU_E_ARG, "set_phase_lock: more locked nodes than nodes");
    cudaSetDevice(h->device);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "set_phase_lock");
    if (h->lock) cudaFree(h->lock);
    h->lock = nullptr;
    h->lock_n = 0;
    if (count > 0) {
        if (cudaMalloc(&h->lock, sizeof(int32_t) * (size_t)count) != cudaSuccess)
            return set_error(h, GLGPU_E_OOM, "set_phase_lock: out of device memory");
        e = cudaMemcpy(h->lock, nodes, sizeof(int32_t) * (size_t)count, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_check(h, e, "set_phase_lock");
        h->lock_n = count;
    }
    drop_td_graphs(h);
    upload_inst(h);
    return cuda_check(h, cudaStreamSynchronize(h->stream), "set_phase_lock");
}

int glgpu_td(glgpu_handle* h, double dt, int32_t Nt, int32_t eqn, glgpu_td_stats* stats) {
    if (check_handle(h)) return GLGPU_E_ARG;
    cudaSetDevice(h->device);
    return td_run(h, dt, Nt, eqn, stats, nullptr);
}

int glgpu_td_timed(glgpu_handle* h, double dt, int32_t Nt, int32_t eqn, glgpu_td_stats* stats, double* elapsed_ms) {
    if (check_handle(h) || !elapsed_ms) return set_error(h, GLGPU_E_ARG, "td_timed: NULL argument");
    cudaSetDevice(h->device);
    return td_run(h, dt, Nt, eqn, stats, elapsed_ms);
}

int glgpu_time_sweeps(glgpu_handle* h, int32_t which, int32_t nrep, double* avg_ms) {
    if (check_handle(h)) return GLGPU_E_ARG;
    cudaSetDevice(h->device);
    return time_sweeps(h, which, nrep, avg_ms);
}

int glgpu_free_energy(glgpu_handle* h, double* energy) {
    if (check_handle(h) || !energy) return set_error(h, GLGPU_E_ARG, "free_energy: NULL argument");
    return obs_free_energy(h, energy);
}

int glgpu_magnetic_field(glgpu_handle* h, void* B) {
    if (check_handle(h) || !B) return set_error(h, GLGPU_E_ARG, "magnetic_field: NULL argument");
    return obs_magnetic_field(h, B);
}

int glgpu_current_density(glgpu_handle* h, void* j) {
    if (check_handle(h) || !j) return set_error(h, GLGPU_E_ARG, "current_density: NULL argument");
    return obs_current_density(h, j);
}

int glgpu_supercurrent_density(glgpu_handle* h, void* js) {
    if (check_handle(h) || !js) return set_error(h, GLGPU_E_ARG, "supercurrent_density: NULL argument");
    return obs_supercurrent_density(h, js);
}

int glgpu_vortex_candidates(glgpu_handle* h, int32_t cap, int32_t* n_out, int32_t* cells, void* corners) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return obs_vortex_candidates(h, cap, n_out, cells, corners);
}

int glgpu_cg_reset_direction(glgpu_handle* h) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return cg_reset_direction(h);
}

int glgpu_cg_gradient(glgpu_handle* h, int32_t compute_beta) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return cg_gradient(h, compute_beta);
}

int glgpu_cg_coefficients(glgpu_handle* h, double* c) {
    if (check_handle(h) || !c) return set_error(h, GLGPU_E_ARG, "cg_coefficients: NULL argument");
    return cg_coefficients(h, c);
}

int glgpu_cg_update(glgpu_handle* h, double alpha_psi, double alpha_A, double* energy) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return cg_update(h, alpha_psi, alpha_A, energy);
}

int glgpu_jacobian(glgpu_handle* h, void* g_psi, void* g_A) {
    if (check_handle(h) || !g_psi) return set_error(h, GLGPU_E_ARG, "jacobian: NULL argument");
    return cg_read_gradient(h, g_psi, g_A);
}

int glgpu_conjgrad_coef(glgpu_handle* h, const void* dpsi, const void* dab, double* c) {
    if (check_handle(h) || !dpsi || !c) return set_error(h, GLGPU_E_ARG, "conjgrad_coef: NULL argument");
    return cg_coef_for(h, dpsi, dab, c);
}

int glgpu_batch_create(glgpu_handle* const* handles, int32_t n, glgpu_batch** out) {
    if (!handles || !out || n < 1) return set_error(nullptr, GLGPU_E_ARG, "glgpu_batch_create: bad arguments");
    *out = nullptr;
    for (int q = 0; q < n; ++q) {
        if (!handles[q]) return set_error(nullptr, GLGPU_E_ARG, "glgpu_batch_create: NULL handle");
        if (handles[q]->dtype != handles[0]->dtype || handles[q]->device != handles[0]->device)
            return set_error(nullptr, GLGPU_E_ARG, "glgpu_batch_create: handles differ in dtype or device");
        for (int r = 0; r < q; ++r)
            if (handles[r] == handles[q]) return set_error(nullptr, GLGPU_E_ARG, "glgpu_batch_create: repeated handle");
    }
    glgpu_batch* b = new glgpu_batch();
    b->dtype = handles[0]->dtype;
    b->device = handles[0]->device;
    b->ninst = n;
    b->hs.assign(handles, handles + n);
    cudaSetDevice(b->device);
    std::vector<Tile> tiles;
    std::vector<ATile> atiles;
    std::vector<Item> items;
    std::vector<const Geo*> geos(n);
    for (int q = 0; q < n; ++q) geos[q] = &handles[q]->g;
    b->strip_rows = choose_strip_rows(b->dtype, geos.data(), n);
    b->inst_items.resize(n);
    for (int q = 0; q < n; ++q) {
        for (int k = 0; k < handles[q]->ntiles; ++k) tiles.push_back(Tile{q, k * kThreads});
        for (int j0 = 0; j0 < handles[q]->g.Ny; j0 += kATY)
            for (int i0 = 0; i0 < handles[q]->g.Nx; i0 += kATX) atiles.push_back(ATile{q, i0, j0, 0});
        const std::vector<Item> it = make_items(handles[q]->g, q, b->strip_rows);
        b->inst_items[q] = strip_items(handles[q]->g.Nx, handles[q]->g.Ny, b->strip_rows);
        items.insert(items.end(), it.begin(), it.end());
    }
    b->ntiles = (int)tiles.size();
    b->natiles = (int)atiles.size();
    b->nitems = (int)items.size();
    b->psi_grid = psi_sweep_grid(psi_kind(b->dtype, 0), b->strip_rows, b->nitems);
    b->gather_h.resize(n);
    bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc(&b->insts, sizeof(Inst) * (size_t)n) == cudaSuccess;
    ok = ok && cudaMalloc(&b->gather, sizeof(InstState) * (size_t)n) == cudaSuccess;
    ok = ok && cudaMalloc(&b->tiles, sizeof(Tile) * tiles.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&b->atiles, sizeof(ATile) * atiles.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&b->items, sizeof(Item) * items.size()) == cudaSuccess;
    ok = ok && cudaMalloc(&b->loop, sizeof(LoopState)) == cudaSuccess;
    ok = ok && cudaMallocHost(&b->gather_pin, sizeof(InstState) * (size_t)n) == cudaSuccess;
    ok = ok && cudaMallocHost(&b->loop_pin, sizeof(LoopState)) == cudaSuccess;
    ok = ok && cudaMallocHost(&b->insts_pin, sizeof(Inst) * (size_t)n) == cudaSuccess;
    cudaError_t e = ok ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->atiles, atiles.data(), sizeof(ATile) * atiles.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->items, items.data(), sizeof(Item) * items.size(), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        glgpu_batch_destroy(b);
        return set_error(nullptr, e == cudaErrorMemoryAllocation ? GLGPU_E_OOM : GLGPU_E_CUDA,
                         std::string("glgpu_batch_create: ") + cudaGetErrorString(e));
    }
    *out = b;
    return GLGPU_OK;
}

int glgpu_batch_destroy(glgpu_batch* b) {
    if (!b) return GLGPU_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (int q = 0; q < kTDGraphs; ++q)
        if (b->td_exec[q]) cudaGraphExecDestroy(b->td_exec[q]);
    if (b->cg_exec) cudaGraphExecDestroy(b->cg_exec);
    void* ptrs[] = {b->insts, b->gather, b->tiles, b->atiles, b->items, b->loop, b->cg_partials, b->cg_loop, b->cg_tiles};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    void* pins[] = {b->gather_pin, b->loop_pin, b->insts_pin};
    for (void* p : pins)
        if (p) cudaFreeHost(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GLGPU_OK;
}

const char* glgpu_batch_last_error(const glgpu_batch* b) { return b ? b->last_error.c_str() : g_create_error.c_str(); }

int glgpu_batch_td(glgpu_batch* b, double dt, int32_t Nt, int32_t eqn, glgpu_td_stats* stats, double* elapsed_ms) {
    if (!b) return GLGPU_E_ARG;
    cudaSetDevice(b->device);
    return batch_td(b, dt, Nt, eqn, stats, elapsed_ms);
}

int glgpu_batch_cg(glgpu_batch* b, int32_t n_iter, double rtol, double gtol, int32_t flags, int32_t* iters,
                   double* energies, double* grad_rel, int32_t* status, double* elapsed_ms) {
    if (!b) return GLGPU_E_ARG;
    cudaSetDevice(b->device);
    return batch_cg(b, n_iter, rtol, gtol, flags, iters, energies, grad_rel, status, elapsed_ms);
}

int glgpu_batch_set_cg_window(glgpu_batch* b, int32_t window, double rel_tol) {
    if (!b) return GLGPU_E_ARG;
    return batch_set_cg_window(b, window, rel_tol);
}

int glgpu_batch_set_energy_targets(glgpu_batch* b, const double* targets, double rel_tol) {
    if (!b) return GLGPU_E_ARG;
    return batch_set_energy_targets(b, targets, rel_tol);
}

int glgpu_batch_set_use_graphs(glgpu_batch* b, int32_t enable) {
    if (!b) return GLGPU_E_ARG;
    b->use_graphs = enable != 0;
    return GLGPU_OK;
}

int glgpu_batch_set_loop_guard(glgpu_batch* b, int32_t launches) {
    if (!b) return GLGPU_E_ARG;
    if (launches < 0) return batch_error(b, GLGPU_E_ARG, "batch_set_loop_guard: launches must be >= 0");
    b->loop_guard = launches;
    return GLGPU_OK;
}

int glgpu_free_energy_noalloc(const glgpu_grid* grid, const glgpu_params* params, const void* psi, const void* ab,
                              const void* abei, const uint8_t* mt, double* energy, void* stream) {
    return free_energy_noalloc(grid, params, psi, ab, abei, mt, energy, (cudaStream_t)stream);
}

int glgpu_reduce_sum(glgpu_handle* h, const double* x, int64_t n, int32_t nv, double* out) {
    if (check_handle(h)) return GLGPU_E_ARG;
    return reduce_sum(h, x, (long long)n, nv, out);
}

}  // extern "C"
