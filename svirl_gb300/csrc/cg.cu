// Modified nonlinear conjugate gradient of the GL free energy, in fused phases:
//   k_cg_grad:      dF/dpsi and dF/dA (svirl/cuda/cg.h:15-301) plus the four
//                   Polak-Ribiere sums (svirl/cuda/utils.h:12-70);
//   k_cg_beta:      beta = max(num/den, 0) (svirl/solvers/cg.py:422-449,
//                   svirl/cuda/utils.h:139-146);
//   k_cg_dir_coef:  dir = beta*dir - g (svirl/cuda/utils.h:96-114) and the 5 or 17
//                   line-search coefficients (svirl/cuda/cg.h:314-731) in one pass,
//                   neighbour directions recomputed in registers;
//   k_cg_update:    psi += a_psi dir, A += a_A dir_A (svirl/cuda/utils.h:73-92).
// All sums accumulate in FP64 and finish in the launch's last CTA.  These are
// the single-instance kernels of the reference-decision CG (step length chosen
// on the host); the batched device CG is in cgb.cu.
#include "glgpu_internal.h"
#include "glgpu_phys.cuh"

namespace glgpu {

// Gradient at node n (psi part) and its two links (A part), plus the four
// Polak-Ribiere sums.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_cg_grad(Geo g, double kappa2, double eps0, const T* eps_sp, double H, const uint8_t* mt,
          const C2<T>* __restrict__ psi, const T* abei, const T* ab,
          C2<T>* __restrict__ gpsi, T* __restrict__ gA, const C2<T>* __restrict__ gpsi_prev, const T* __restrict__ gA_prev,
          int solveA, double* partials, unsigned* counter, double* dscal) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    T v[4] = {T(0), T(0), T(0), T(0)};
    if (n < g.N) {
        const int i = n % g.Nx, j = n / g.Nx;
        const unsigned cb = cell_bits(g, mt, i, j);
        const C2<T> G = grad_psi_node<T>(g, (T)eps0, eps_sp, psi, PhaseLinks<T>{abei, ab}, n, i, j, cb);
        gpsi[n] = G;
        const C2<T> Gp = gpsi_prev[n];
        v[0] = G.x * (G.x - Gp.x) + G.y * (G.y - Gp.y);
        v[1] = Gp.x * Gp.x + Gp.y * Gp.y;
        if (solveA) {
            const T k2 = (T)kappa2, Hh = (T)H;
            if (i < g.Nx - 1) {
                const int na = i + (g.Nx - 1) * j;
                const T Ga = grad_A_link<T>(g, k2, Hh, psi, abei, ab, PhaseLinks<T>{abei, ab}, n, i, j, cb, true);
                gA[na] = Ga;
                const T Gpa = gA_prev[na];
                v[2] += Ga * (Ga - Gpa);
                v[3] += Gpa * Gpa;
            }
            if (j < g.Ny - 1) {
                const int nb = g.Na + i + g.Nx * j;
                const T Gb = grad_A_link<T>(g, k2, Hh, psi, abei, ab, PhaseLinks<T>{abei, ab}, n, i, j, cb, false);
                gA[nb] = Gb;
                const T Gpb = gA_prev[nb];
                v[2] += Gb * (Gb - Gpb);
                v[3] += Gpb * Gpb;
            }
        }
    }
    grid_sum_finish(v, partials, counter, dscal + 24, 1.0);
}

// beta = max(num/den, 0) with the reference's float semantics (divide_scalars_positive).
template <typename T>
__global__ void k_cg_beta(double* dscal, int solveA) {
    if (threadIdx.x != 0) return;
    T q = (T)dscal[24] / (T)dscal[25];
    dscal[28] = (double)fmax(q, T(0));
    if (solveA) {
        T qa = (T)dscal[26] / (T)dscal[27];
        dscal[29] = (double)fmax(qa, T(0));
    }
}

// Direction update and line-search coefficients.  NV = 5: F(psi + a dpsi)
// (cg.h:314-474); NV = 17: F(psi + a_psi dpsi, A + a_A dA) (cg.h:477-731).
// dir_mode 1: d = beta*dO - g, stored into dN; dir_mode 0: d = dO as given.
template <typename T, int NV>
__global__ void __launch_bounds__(kThreads)
k_cg_dir_coef(Geo g, double kappa2, double eps0, const T* eps_sp, double H, const uint8_t* mt,
              const C2<T>* __restrict__ psi, const T* abei, const T* ab,
              const C2<T>* __restrict__ gpsi, const T* __restrict__ gA,
              const C2<T>* __restrict__ dO, const T* __restrict__ dAO,
              C2<T>* __restrict__ dN, T* __restrict__ dAN, int dir_mode,
              double* partials, unsigned* counter, double* dscal) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    T c[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) c[k] = T(0);
    const T bp = (T)dscal[28], bA = (T)dscal[29];
    auto dpsi = [&](int m) -> C2<T> {
        const C2<T> o = dO[m];
        if (!dir_mode) return o;
        const C2<T> gg = gpsi[m];
        return cmk<T>(bp * o.x - gg.x, bp * o.y - gg.y);
    };
    auto dA = [&](int m) -> T {
        const T o = dAO[m];
        if (!dir_mode) return o;
        return bA * o - gA[m];
    };
    if (n < g.N) {
        const int i = n % g.Nx, j = n / g.Nx;
        const unsigned cb = cell_bits(g, mt, i, j);
        if (dir_mode) {
            dN[n] = dpsi(n);
            if (NV == 17) {
                if (i < g.Nx - 1) { int na = i + (g.Nx - 1) * j; dAN[na] = dA(na); }
                if (j < g.Ny - 1) { int nb = g.Na + i + g.Nx * j; dAN[nb] = dA(nb); }
            }
        }
        coef_node<T, NV>(g, (T)kappa2, (T)eps0, eps_sp, (T)H, [psi](int m) { return psi[m]; },
                         [abei, ab](int l) { return link_phase(abei, ab, l); }, ab, PhaseLinks<T>{abei, ab}, n, i, j, cb,
                         dpsi, dA, c);
    }
    grid_sum_finish(c, partials, counter, dscal, g.dxdy);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_cg_update(Geo g, C2<T>* __restrict__ psi, T* __restrict__ ab, const C2<T>* __restrict__ dpsi, const T* __restrict__ dA,
            T a_psi, T a_A, int solveA) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    if (n >= g.N) return;
    const C2<T> d = dpsi[n];
    C2<T> p = psi[n];
    p.x = a_psi * d.x + p.x;
    p.y = a_psi * d.y + p.y;
    psi[n] = p;
    if (solveA) {
        const int i = n % g.Nx, j = n / g.Nx;
        if (i < g.Nx - 1) { int na = i + (g.Nx - 1) * j; ab[na] = a_A * dA[na] + ab[na]; }
        if (j < g.Ny - 1) { int nb = g.Na + i + g.Nx * j; ab[nb] = a_A * dA[nb] + ab[nb]; }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

int obs_free_energy(glgpu_handle* h, double* out);

static inline bool fk(const glgpu_handle* h) { return h->p.kappa > 0.0 && !std::isinf(h->p.kappa); }
static inline double k2(const glgpu_handle* h) { return fk(h) ? h->p.kappa * h->p.kappa : -1.0; }

int cg_ensure(glgpu_handle* h) {
    if (h->g_psi[0]) return GLGPU_OK;
    const size_t cb = (size_t)h->g.N * 2 * real_size(h), ab = (size_t)h->g.Nab * real_size(h);
    for (int q = 0; q < 2; ++q) {
        if (cudaMalloc(&h->g_psi[q], cb) != cudaSuccess || cudaMalloc(&h->dir_psi[q], cb) != cudaSuccess ||
            cudaMalloc(&h->g_A[q], ab) != cudaSuccess || cudaMalloc(&h->dir_A[q], ab) != cudaSuccess)
            return set_error(h, GLGPU_E_OOM, "cg: out of device memory");
        cudaMemsetAsync(h->g_psi[q], 0, cb, h->stream);
        cudaMemsetAsync(h->dir_psi[q], 0, cb, h->stream);
        cudaMemsetAsync(h->g_A[q], 0, ab, h->stream);
        cudaMemsetAsync(h->dir_A[q], 0, ab, h->stream);
    }
    cudaMemsetAsync(h->dscal + 28, 0, 2 * sizeof(double), h->stream);  // beta = 0
    if (cudaMalloc(&h->cgst, sizeof(CGState)) != cudaSuccess || cudaMalloc(&h->cbits, (size_t)h->g.N) != cudaSuccess)
        return set_error(h, GLGPU_E_OOM, "cg: out of device memory");
    cudaMemsetAsync(h->cgst, 0, sizeof(CGState), h->stream);
    h->cg_g = 0;
    h->cg_dir = 0;
    upload_inst(h);  // the descriptor carries the CG buffers
    return cuda_check(h, cudaStreamSynchronize(h->stream), "cg_ensure");
}

int cg_reset_direction(glgpu_handle* h) {
    int rc = cg_ensure(h);
    if (rc) return rc;
    return cuda_check(h, cudaMemsetAsync(h->dir_psi[h->cg_dir], 0, (size_t)h->g.N * 2 * real_size(h), h->stream), "cg_reset_direction");
}

template <typename T>
static void launch_grad(glgpu_handle* h, int out_idx, int beta) {
    const int prev = 1 - out_idx;
    k_cg_grad<T><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(
        h->g, k2(h), h->p.epsilon, (const T*)h->eps_sp, h->p.H, h->mt, (const C2<T>*)h->psi[0], (const T*)h->abei, (const T*)h->ab[0],
        (C2<T>*)h->g_psi[out_idx], (T*)h->g_A[out_idx], (const C2<T>*)h->g_psi[prev], (const T*)h->g_A[prev], fk(h) ? 1 : 0,
        h->partials, h->counter, h->dscal);
    if (beta) k_cg_beta<T><<<1, 32, 0, h->stream>>>(h->dscal, fk(h) ? 1 : 0);
}

int cg_gradient(glgpu_handle* h, int compute_beta) {
    int rc = cg_ensure(h);
    if (rc) return rc;
    const int out_idx = 1 - h->cg_g;
    if (h->dtype == 8) launch_grad<double>(h, out_idx, compute_beta);
    else launch_grad<float>(h, out_idx, compute_beta);
    h->cg_g = out_idx;
    return cuda_check(h, cudaGetLastError(), "cg_gradient");
}

template <typename T, int NV>
static void launch_coef(glgpu_handle* h, const void* dO, const void* dAO, void* dN, void* dAN, int dir_mode) {
    k_cg_dir_coef<T, NV><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(
        h->g, k2(h), h->p.epsilon, (const T*)h->eps_sp, h->p.H, h->mt, (const C2<T>*)h->psi[0], (const T*)h->abei, (const T*)h->ab[0],
        (const C2<T>*)h->g_psi[h->cg_g], (const T*)h->g_A[h->cg_g], (const C2<T>*)dO, (const T*)dAO, (C2<T>*)dN, (T*)dAN, dir_mode,
        h->partials, h->counter, h->dscal);
}

static int read_coefs(glgpu_handle* h, double* c, int nv) {
    cudaError_t e = cudaMemcpyAsync(h->hscal, h->dscal, nv * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "cg coefficients");
    for (int k = 0; k < nv; ++k) c[k] = h->hscal[k];
    return GLGPU_OK;
}

int cg_coefficients(glgpu_handle* h, double* c_out) {
    int rc = cg_ensure(h);
    if (rc) return rc;
    const int o = h->cg_dir, nw = 1 - o;
    const bool A = fk(h);
    if (h->dtype == 8) {
        if (A) launch_coef<double, 17>(h, h->dir_psi[o], h->dir_A[o], h->dir_psi[nw], h->dir_A[nw], 1);
        else launch_coef<double, 5>(h, h->dir_psi[o], h->dir_A[o], h->dir_psi[nw], h->dir_A[nw], 1);
    } else {
        if (A) launch_coef<float, 17>(h, h->dir_psi[o], h->dir_A[o], h->dir_psi[nw], h->dir_A[nw], 1);
        else launch_coef<float, 5>(h, h->dir_psi[o], h->dir_A[o], h->dir_psi[nw], h->dir_A[nw], 1);
    }
    h->cg_dir = nw;
    rc = cuda_check(h, cudaGetLastError(), "cg_coefficients");
    if (rc) return rc;
    return read_coefs(h, c_out, A ? 17 : 5);
}

int cg_update(glgpu_handle* h, double alpha_psi, double alpha_A, double* energy_out) {
    int rc = cg_ensure(h);
    if (rc) return rc;
    const int d = h->cg_dir;
    if (h->dtype == 8)
        k_cg_update<double><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(h->g, (double2*)h->psi[0], (double*)h->ab[0],
                                                                           (const double2*)h->dir_psi[d], (const double*)h->dir_A[d],
                                                                           alpha_psi, alpha_A, fk(h) ? 1 : 0);
    else
        k_cg_update<float><<<blocks_for(h->g.N), kThreads, 0, h->stream>>>(h->g, (float2*)h->psi[0], (float*)h->ab[0],
                                                                          (const float2*)h->dir_psi[d], (const float*)h->dir_A[d],
                                                                          (float)alpha_psi, (float)alpha_A, fk(h) ? 1 : 0);
    rc = cuda_check(h, cudaGetLastError(), "cg_update");
    if (rc) return rc;
    if (energy_out) return obs_free_energy(h, energy_out);
    return GLGPU_OK;
}

int cg_read_gradient(glgpu_handle* h, void* gpsi_host, void* gA_host) {
    int rc = cg_ensure(h);
    if (rc) return rc;
    // evaluate into the spare buffer without touching the CG state
    const int spare = 1 - h->cg_g;
    if (h->dtype == 8) launch_grad<double>(h, spare, 0);
    else launch_grad<float>(h, spare, 0);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && gpsi_host)
        e = cudaMemcpyAsync(gpsi_host, h->g_psi[spare], (size_t)h->g.N * 2 * real_size(h), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && gA_host)
        e = cudaMemcpyAsync(gA_host, h->g_A[spare], (size_t)h->g.Nab * real_size(h), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return cuda_check(h, e, "jacobian");
}

int cg_coef_for(glgpu_handle* h, const void* dpsi_host, const void* dab_host, double* c_out) {
    int rc = cg_ensure(h);
    if (rc) return rc;
    const int spare = 1 - h->cg_dir;
    cudaError_t e = cudaMemcpyAsync(h->dir_psi[spare], dpsi_host, (size_t)h->g.N * 2 * real_size(h), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && dab_host)
        e = cudaMemcpyAsync(h->dir_A[spare], dab_host, (size_t)h->g.Nab * real_size(h), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "conjgrad_coef upload");
    const bool A = dab_host != nullptr;
    if (h->dtype == 8) {
        if (A) launch_coef<double, 17>(h, h->dir_psi[spare], h->dir_A[spare], nullptr, nullptr, 0);
        else launch_coef<double, 5>(h, h->dir_psi[spare], h->dir_A[spare], nullptr, nullptr, 0);
    } else {
        if (A) launch_coef<float, 17>(h, h->dir_psi[spare], h->dir_A[spare], nullptr, nullptr, 0);
        else launch_coef<float, 5>(h, h->dir_psi[spare], h->dir_A[spare], nullptr, nullptr, 0);
    }
    rc = cuda_check(h, cudaGetLastError(), "conjgrad_coef");
    if (rc) return rc;
    return read_coefs(h, c_out, A ? 17 : 5);
}

}  // namespace glgpu
