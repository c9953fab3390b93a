// Modified nonlinear conjugate gradient of the GL free energy, in fused phases:
//   k_cg_grad:      dF/dpsi and dF/dA (svirl/cuda/cg.h:15-301) plus the four
//                   Polak-Ribiere sums and beta = max(num/den, 0)
//                   (svirl/solvers/cg.py:422-449, svirl/cuda/utils.h:12-70,139-146);
//   k_cg_dir_coef:  dir = beta*dir - g (svirl/cuda/utils.h:96-114) and the 5 or 17
//                   line-search coefficients (svirl/cuda/cg.h:314-731) in one pass,
//                   neighbour directions recomputed in registers;
//   k_cg_update:    psi += a_psi dir, A += a_A dir_A (svirl/cuda/utils.h:73-92).
// All sums accumulate in FP64 and finish in the launch's last CTA.
#include "glgpu_internal.h"

namespace glgpu {

template <typename T> struct DuW2 {
    T r_m0, r_p0, r_0m, r_0p, g;
};
template <typename T> __device__ __forceinline__ DuW2<T> du_w(unsigned cb) {
    DuW2<T> w;
    const T mm = GL_MM(cb) ? T(1) : T(0), mp = GL_MP(cb) ? T(1) : T(0);
    const T pm = GL_PM(cb) ? T(1) : T(0), pp = GL_PP(cb) ? T(1) : T(0);
    w.r_m0 = T(0.5) * (mm + mp);
    w.r_p0 = T(0.5) * (pm + pp);
    w.r_0m = T(0.5) * (mm + pm);
    w.r_0p = T(0.5) * (mp + pp);
    w.g = T(0.25) * (w.r_m0 + w.r_p0 + w.r_0m + w.r_0p);
    return w;
}

template <typename T> __device__ __forceinline__ T lphase(const T* abei, const T* ab, int n) {
    T p = T(0);
    if (abei) p += abei[n];
    if (ab) p += ab[n];
    return p;
}

// 2 (psi0 - psi1 U(ph)) (svirl/cuda/cg.h:4-12)
template <typename T> __device__ __forceinline__ C2<T> gjac(C2<T> p0, T ph, C2<T> p1) {
    T s, c;
    sincos_t(ph, &s, &c);
    return cmk<T>(T(2) * (p0.x - (p1.x * c + p1.y * s)), T(2) * (p0.y - (p1.y * c - p1.x * s)));
}

template <typename T>
__device__ __forceinline__ T curlcurl_grad(const Geo& g, const T* abei, const T* ab, T H, int i, int j, bool xdir) {
    const int Nxa = g.Nx - 1, Na = g.Na, Nx = g.Nx;
    const T idx = GT(g, idx), idy = GT(g, idy);
    const T idx2 = GT(g, idx2), idy2 = GT(g, idy2), idxy = GT(g, idxy);
    T c = T(0), dd = T(1);
    if (xdir) {
        const int n = i + Nxa * j;
        if (j == 0) { c -= T(2) * H * idy; dd = T(2); }
        else if (j + 1 == g.Ny) { c += T(2) * H * idy; dd = T(2); }
        if (abei) c += T(2) / dd * idy2 * abei[n];
        if (ab) c += T(2) * idy2 * ab[n];
        if (j > 0) {
            if (abei) c += (-idy2 * abei[i + Nxa * (j - 1)] + idxy * abei[Na + i + Nx * (j - 1)] - idxy * abei[Na + i + 1 + Nx * (j - 1)]);
            if (ab) c += dd * (-idy2 * ab[i + Nxa * (j - 1)] + idxy * ab[Na + i + Nx * (j - 1)] - idxy * ab[Na + i + 1 + Nx * (j - 1)]);
        }
        if (j + 1 < g.Ny) {
            if (abei) c += (-idy2 * abei[i + Nxa * (j + 1)] - idxy * abei[Na + i + Nx * j] + idxy * abei[Na + i + 1 + Nx * j]);
            if (ab) c += dd * (-idy2 * ab[i + Nxa * (j + 1)] - idxy * ab[Na + i + Nx * j] + idxy * ab[Na + i + 1 + Nx * j]);
        }
    } else {
        const int n = Na + i + Nx * j;
        if (i == 0) { c += T(2) * H * idx; dd = T(2); }
        else if (i + 1 == g.Nx) { c -= T(2) * H * idx; dd = T(2); }
        if (abei) c += T(2) / dd * idx2 * abei[n];
        if (ab) c += T(2) * idx2 * ab[n];
        if (i > 0) {
            if (abei) c += (-idx2 * abei[Na + (i - 1) + Nx * j] + idxy * abei[(i - 1) + Nxa * j] - idxy * abei[(i - 1) + Nxa * (j + 1)]);
            if (ab) c += dd * (-idx2 * ab[Na + (i - 1) + Nx * j] + idxy * ab[(i - 1) + Nxa * j] - idxy * ab[(i - 1) + Nxa * (j + 1)]);
        }
        if (i + 1 < g.Nx) {
            if (abei) c += (-idx2 * abei[Na + (i + 1) + Nx * j] - idxy * abei[i + Nxa * j] + idxy * abei[i + Nxa * (j + 1)]);
            if (ab) c += dd * (-idx2 * ab[Na + (i + 1) + Nx * j] - idxy * ab[i + Nxa * j] + idxy * ab[i + Nxa * (j + 1)]);
        }
    }
    return c;
}

// Gradient at node n (psi part) and its two links (A part), plus the four
// Polak-Ribiere sums.  beta_mode: 0 = gradient only, 1 = also update beta.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_cg_grad(Geo g, double kappa2, double eps0, const T* eps_sp, double H, const uint8_t* mt,
          const C2<T>* __restrict__ psi, const T* abei, const T* ab,
          C2<T>* __restrict__ gpsi, T* __restrict__ gA, const C2<T>* __restrict__ gpsi_prev, const T* __restrict__ gA_prev,
          int solveA, int beta_mode, double* partials, unsigned* counter, double* dscal) {
    const int n = blockIdx.x * kThreads + threadIdx.x;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (n < g.N) {
        const int i = n % g.Nx, j = n / g.Nx;
        const unsigned cb = cell_bits(g, mt, i, j);
        const T dx = GT(g, dx), dy = GT(g, dy), idx = GT(g, idx), idy = GT(g, idy);
        const T idx2 = GT(g, idx2), idy2 = GT(g, idy2);
        const C2<T> p0 = psi[n];
        C2<T> gj = cmk<T>(T(0), T(0));
        if (cb) {
            const DuW2<T> w = du_w<T>(cb);
            const T eps = eps_sp ? eps_sp[n] : (T)eps0;
            const T p = p0.x * p0.x + p0.y * p0.y - eps;
            gj = cadd(gj, cscale(T(2) * w.g * p, p0));
            if (GL_MM(cb) || GL_MP(cb))
                gj = cadd(gj, cscale(w.r_m0 * idx2, gjac<T>(p0, -dx * lphase(abei, ab, (i - 1) + (g.Nx - 1) * j), psi[n - 1])));
            if (GL_PM(cb) || GL_PP(cb))
                gj = cadd(gj, cscale(w.r_p0 * idx2, gjac<T>(p0, dx * lphase(abei, ab, i + (g.Nx - 1) * j), psi[n + 1])));
            if (GL_MM(cb) || GL_PM(cb))
                gj = cadd(gj, cscale(w.r_0m * idy2, gjac<T>(p0, -dy * lphase(abei, ab, g.Na + i + g.Nx * (j - 1)), psi[n - g.Nx])));
            if (GL_MP(cb) || GL_PP(cb))
                gj = cadd(gj, cscale(w.r_0p * idy2, gjac<T>(p0, dy * lphase(abei, ab, g.Na + i + g.Nx * j), psi[n + g.Nx])));
        }
        const T dxdy = dx * dy;
        const C2<T> G = cscale(dxdy, gj);
        gpsi[n] = G;
        const C2<T> Gp = gpsi_prev[n];
        v[0] = (double)(G.x * (G.x - Gp.x) + G.y * (G.y - Gp.y));
        v[1] = (double)(Gp.x * Gp.x + Gp.y * Gp.y);
        if (solveA) {
            const T k2 = (T)kappa2, Hh = (T)H;
            if (i < g.Nx - 1) {
                const int na = i + (g.Nx - 1) * j;
                T c = k2 * curlcurl_grad<T>(g, abei, ab, Hh, i, j, true);
                if (GL_PM(cb) || GL_PP(cb)) {
                    const T r = T(0.5) * ((GL_PM(cb) ? T(1) : T(0)) + (GL_PP(cb) ? T(1) : T(0)));
                    c += -r * idx * js_of<T>(p0, dx * lphase(abei, ab, na), psi[n + 1]);
                }
                const T Ga = T(2) * dxdy * c;
                gA[na] = Ga;
                const T Gpa = gA_prev[na];
                v[2] += (double)(Ga * (Ga - Gpa));
                v[3] += (double)(Gpa * Gpa);
            }
            if (j < g.Ny - 1) {
                const int nb = g.Na + i + g.Nx * j;
                T c = k2 * curlcurl_grad<T>(g, abei, ab, Hh, i, j, false);
                if (GL_MP(cb) || GL_PP(cb)) {
                    const T r = T(0.5) * ((GL_MP(cb) ? T(1) : T(0)) + (GL_PP(cb) ? T(1) : T(0)));
                    c += -r * idy * js_of<T>(p0, dy * lphase(abei, ab, nb), psi[n + g.Nx]);
                }
                const T Gb = T(2) * dxdy * c;
                gA[nb] = Gb;
                const T Gpb = gA_prev[nb];
                v[2] += (double)(Gb * (Gb - Gpb));
                v[3] += (double)(Gpb * Gpb);
            }
        }
    }
    grid_sum_finish<4>(v, partials, counter, dscal + 24, 1.0);
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
    double c[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) c[k] = 0.0;
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
        const T dx = GT(g, dx), dy = GT(g, dy), idx = GT(g, idx), idy = GT(g, idy);
        const T idx2 = GT(g, idx2), idy2 = GT(g, idy2);
        const C2<T> d0 = dpsi(n);
        if (dir_mode) dN[n] = d0;
        if (NV == 17 && dir_mode) {
            if (i < g.Nx - 1) { int na = i + (g.Nx - 1) * j; dAN[na] = dA(na); }
            if (j < g.Ny - 1) { int nb = g.Na + i + g.Nx * j; dAN[nb] = dA(nb); }
        }
        if (cb) {
            const DuW2<T> w = du_w<T>(cb);
            const C2<T> p0 = psi[n];
            const T eps = eps_sp ? eps_sp[n] : (T)eps0;
            const T p2 = cabs2(p0), d2 = cabs2(d0);
            const T tw = T(2) * (p0.x * d0.x + p0.y * d0.y);
            const T k00 = w.g * (T(0.5) * p2 - eps) * p2;
            const T k10 = w.g * tw * (p2 - eps);
            const T k20 = w.g * (-eps * d2 + T(0.5) * tw * tw + p2 * d2);
            const T k30 = w.g * tw * d2;
            const T k40 = w.g * T(0.5) * d2 * d2;
            if (NV == 5) {
                c[0] += k00; c[1] += k10; c[2] += k20; c[3] += k30; c[4] += k40;
            } else {
                c[0] += k00; c[5] += k10; c[10] += k20; c[15] += k30; c[16] += k40;
            }
#pragma unroll
            for (int dir = 0; dir < 2; ++dir) {
                const bool on = dir == 0 ? (GL_PM(cb) || GL_PP(cb)) : (GL_MP(cb) || GL_PP(cb));
                if (!on) continue;
                const int nl = dir == 0 ? i + (g.Nx - 1) * j : g.Na + i + g.Nx * j;
                const int m1 = dir == 0 ? n + 1 : n + g.Nx;
                const T d = dir == 0 ? dx : dy;
                const T wr = (dir == 0 ? w.r_p0 : w.r_0p) * (dir == 0 ? idx2 : idy2);
                T ph = T(0);
                if (abei) ph += d * abei[nl];
                if (ab) ph += d * ab[nl];
                const C2<T> p1 = psi[m1], d1 = dpsi(m1);
                T s, cs;
                sincos_t(ph, &s, &cs);
                const C2<T> gp = grad_c_sc<T>(p0, s, cs, p1), gd = grad_c_sc<T>(d0, s, cs, d1);
                const T gg_p = gp.x * gp.x + gp.y * gp.y;
                const T gg_d = gd.x * gd.x + gd.y * gd.y;
                const T zr = gp.x * gd.x + gp.y * gd.y;   // Re(conj(gp) * gd)
                if (NV == 5) {
                    c[2] += wr * gg_d;
                    c[1] += wr * T(2) * zr;
                    c[0] += wr * gg_p;
                } else {
                    c[0] += wr * gg_p;
                    c[5] += wr * T(2) * zr;
                    c[10] += wr * gg_d;
                    const T dph = d * dA(nl);
                    const T dph2 = dph * dph;
                    // U(-ph) = (cos ph, sin ph)
                    const C2<T> Um = cmk<T>(cs, s);
                    const C2<T> z1 = cmul(cmul(p0, Um), cconj(p1));
                    const C2<T> z2 = cadd(cmul(cmul(p0, Um), cconj(d1)), cmul(cmul(d0, Um), cconj(p1)));
                    const C2<T> z3 = cmul(cmul(d0, Um), cconj(d1));
                    const C2<T> zz[3] = {z1, z2, z3};
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const int b = 1 + 5 * q;
                        c[b + 0] += wr * T(2) * zz[q].y * dph;
                        c[b + 1] += wr * zz[q].x * dph2;
                        c[b + 2] += -wr / T(3) * zz[q].y * dph2 * dph;
                        c[b + 3] += -wr / T(12) * zz[q].x * dph2 * dph2;
                    }
                }
            }
        }
        if (kappa2 > 0.0 && i < g.Nxc && j < g.Nyc) {
            const int Nxa = g.Nx - 1;
            const int ia00 = i + Nxa * j, ia0p = i + Nxa * (j + 1), ib00 = g.Na + i + g.Nx * j, ibp0 = g.Na + i + 1 + g.Nx * j;
            const T k2 = (T)kappa2;
            if (NV == 5) {
                const T dB = idx * (ab[ibp0] - ab[ib00]) - idy * (ab[ia0p] - ab[ia00]) - (T)H;
                c[0] += k2 * dB * dB;
            } else {
                const T a00 = lphase(abei, ab, ia00), a0p = lphase(abei, ab, ia0p);
                const T b00 = lphase(abei, ab, ib00), bp0 = lphase(abei, ab, ibp0);
                const T BH = idx * (bp0 - b00) - idy * (a0p - a00) - (T)H;
                const T dB = idx * (dA(ibp0) - dA(ib00)) - idy * (dA(ia0p) - dA(ia00));
                c[0] += k2 * BH * BH;
                c[1] += k2 * T(2) * BH * dB;
                c[2] += k2 * dB * dB;
            }
        }
    }
    grid_sum_finish<NV>(c, partials, counter, dscal, g.dxdy);
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
    h->cg_g = 0;
    h->cg_dir = 0;
    return cuda_check(h, cudaGetLastError(), "cg_ensure");
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
        (C2<T>*)h->g_psi[out_idx], (T*)h->g_A[out_idx], (const C2<T>*)h->g_psi[prev], (const T*)h->g_A[prev], fk(h) ? 1 : 0, beta,
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
