// Per-node GL physics shared by the observable, single-instance CG and batched
// CG kernels: Du link weights, the free-energy pseudo-density, the gradients
// dF/dpsi and dF/dA, and the line-search polynomial coefficients of one node.
//
// Reference: svirl/cuda/observables.h:238-362 (energy), svirl/cuda/cg.h:4-301
// (gradients), svirl/cuda/cg.h:314-731 (coefficients).
#pragma once

#include "glgpu_common.cuh"

namespace glgpu {

// Du discretisation weights (svirl/cuda/observables.h:294-299).
template <typename T> struct DuW {
    T r_m0, r_p0, r_0m, r_0p, g;
};
template <typename T> __device__ __forceinline__ DuW<T> du_weights(unsigned cb) {
    DuW<T> w;
    const T mm = GL_MM(cb) ? T(1) : T(0), mp = GL_MP(cb) ? T(1) : T(0);
    const T pm = GL_PM(cb) ? T(1) : T(0), pp = GL_PP(cb) ? T(1) : T(0);
    w.r_m0 = T(0.5) * (mm + mp);
    w.r_p0 = T(0.5) * (pm + pp);
    w.r_0m = T(0.5) * (mm + pm);
    w.r_0p = T(0.5) * (mp + pp);
    w.g = T(0.25) * (w.r_m0 + w.r_p0 + w.r_0m + w.r_0p);
    return w;
}

// abei + ab on one link, each term present when its pointer is non-NULL.
template <typename T> __device__ __forceinline__ T link_phase(const T* abei, const T* ab, int n) {
    T p = T(0);
    if (abei) p += abei[n];
    if (ab) p += ab[n];
    return p;
}

// (sin, cos) of the phase d * A of link l, two ways.  PhaseLinks evaluates them
// on the spot from abei + ab, in the two forms the reference's kernels use:
// sc_sum: d * (abei + ab) (observables.h, cg.h:15-301), sc_split: d*abei + d*ab
// (the coefficient kernels, cg.h:410-412).  TableLinks reads a table
// U[l] = exp(-i d A_l) = (cos, -sin) made once per CG iteration by the kernel
// that updates A, so the gradient, coefficient and energy kernels of the batched
// CG do no transcendental math.
template <typename T> struct PhaseLinks {
    const T* abei;
    const T* ab;
    __device__ __forceinline__ void sc_sum(int l, T d, T& s, T& c) const { sincos_t(d * link_phase(abei, ab, l), &s, &c); }
    __device__ __forceinline__ void sc_split(int l, T d, T& s, T& c) const {
        T ph = T(0);
        if (abei) ph += d * abei[l];
        if (ab) ph += d * ab[l];
        sincos_t(ph, &s, &c);
    }
};
template <typename T> struct TableLinks {
    const C2<T>* U;
    __device__ __forceinline__ void sc_sum(int l, T, T& s, T& c) const {
        const C2<T> u = U[l];
        c = u.x;
        s = -u.y;
    }
    __device__ __forceinline__ void sc_split(int l, T d, T& s, T& c) const { sc_sum(l, d, s, c); }
};

// curl of one link field on cell (i, j): idx*(b[i+1,j]-b[i,j]) - idy*(a[i,j+1]-a[i,j]);
// A(l) gives link l's value.
template <typename T, typename AF>
__device__ __forceinline__ T cell_curl_f(const Geo& g, const AF& A, int i, int j, T idx, T idy) {
    const int Nxa = g.Nx - 1;
    return idx * (A(g.Na + (i + 1) + g.Nx * j) - A(g.Na + i + g.Nx * j)) - idy * (A(i + Nxa * (j + 1)) - A(i + Nxa * j));
}
template <typename T> __device__ __forceinline__ T cell_curl(const Geo& g, const T* A, int i, int j, T idx, T idy) {
    return cell_curl_f<T>(g, [A](int l) { return A[l]; }, i, j, idx, idy);
}

// Free-energy pseudo-density at node n = (i, j) with cell bits cb before the
// dx*dy factor (svirl/cuda/observables.h:276-356).  psi(m) gives the order
// parameter at node m, ab(l) the vector potential of link l (used only when has_ab).
template <typename T, typename LK, typename PF, typename AF>
__device__ __forceinline__ T energy_density_f(const Geo& g, T kappa2, T eps0, const T* eps_sp, T H, unsigned cb,
                                              const PF& psi, const T* abei, bool has_ab, const AF& ab, const LK& lk,
                                              int n, int i, int j) {
    const T dx = GT(g, dx), dy = GT(g, dy), idx = GT(g, idx), idy = GT(g, idy);
    const T idx2 = GT(g, idx2), idy2 = GT(g, idy2);
    T e = T(0);
    if (cb) {
        const DuW<T> w = du_weights<T>(cb);
        const C2<T> p00 = psi(n);
        const T p2 = cabs2(p00);
        const T eps = eps_sp ? eps_sp[n] : eps0;
        e += w.g * (T(0.5) * p2 - eps) * p2;
        if (GL_PM(cb) || GL_PP(cb)) {
            T sn, cs;
            lk.sc_sum(i + (g.Nx - 1) * j, dx, sn, cs);
            const C2<T> gr = grad_c_sc<T>(p00, sn, cs, psi(n + 1));
            e += w.r_p0 * idx2 * (gr.x * gr.x + gr.y * gr.y);
        }
        if (GL_MP(cb) || GL_PP(cb)) {
            T sn, cs;
            lk.sc_sum(g.Na + i + g.Nx * j, dy, sn, cs);
            const C2<T> gr = grad_c_sc<T>(p00, sn, cs, psi(n + g.Nx));
            e += w.r_0p * idy2 * (gr.x * gr.x + gr.y * gr.y);
        }
    }
    if (kappa2 > T(0) && i < g.Nxc && j < g.Nyc) {
        T dB = -H;
        if (abei) dB += cell_curl(g, abei, i, j, idx, idy);
        if (has_ab) dB += cell_curl_f<T>(g, ab, i, j, idx, idy);
        e += kappa2 * dB * dB;
    }
    return e;
}
template <typename T, typename LK>
__device__ __forceinline__ T energy_density(const Geo& g, T kappa2, T eps0, const T* eps_sp, T H,
                                            const uint8_t* mt, const C2<T>* psi, const T* abei, const T* ab,
                                            const LK& lk, int n) {
    const int i = n % g.Nx, j = n / g.Nx;
    return energy_density_f<T>(g, kappa2, eps0, eps_sp, H, cell_bits(g, mt, i, j), [psi](int m) { return psi[m]; },
                               abei, ab != nullptr, [ab](int l) { return ab[l]; }, lk, n, i, j);
}

// curl curl A (times 1/kappa^2) on the link starting at node (i, j) along x (xdir)
// or y, with the reference's boundary terms: the field H and the doubled
// neighbour terms of the A part (dd) at the no-current boundaries
// (svirl/cuda/observables.h:66-155, svirl/cuda/cg.h:174-300).
template <typename T>
__device__ __forceinline__ T curlcurl_link(const Geo& g, const T* abei, const T* ab, T H, int i, int j, bool xdir) {
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

// The exact derivative of the magnetic energy kappa^2 sum_cells (curl A - H)^2
// (before the 2 kappa^2 dx dy factor) on a link of the boundary rows/columns,
// which belongs to one cell only.  The reference's formula above doubles the
// H and ab terms there (the ghost-cell form of the TD equation), so its dF/dA
// does not vanish at the energy minimum on those links; an interior link is the
// same in both.
template <typename T>
__device__ __forceinline__ T curlcurl_link_exact(const Geo& g, const T* abei, const T* ab, T H, int i, int j, bool xdir) {
    const int Nxa = g.Nx - 1, Na = g.Na, Nx = g.Nx;
    const T idx = GT(g, idx), idy = GT(g, idy);
    const T idx2 = GT(g, idx2), idy2 = GT(g, idy2), idxy = GT(g, idxy);
    auto A = [&](int n) -> T { return link_phase(abei, ab, n); };
    if (xdir) {
        if (j == 0)  // cell (i, 0) above the link
            return idy2 * (A(i) - A(i + Nxa)) + idxy * (A(Na + i + 1) - A(Na + i)) - H * idy;
        if (j + 1 == g.Ny)  // cell (i, Ny-2) below the link
            return idy2 * (A(i + Nxa * j) - A(i + Nxa * (j - 1))) - idxy * (A(Na + i + 1 + Nx * (j - 1)) - A(Na + i + Nx * (j - 1))) + H * idy;
    } else {
        if (i == 0)  // cell (0, j) to the right of the link
            return idx2 * (A(Na + Nx * j) - A(Na + 1 + Nx * j)) + idxy * (A(Nxa * (j + 1)) - A(Nxa * j)) + H * idx;
        if (i + 1 == g.Nx)  // cell (Nx-2, j) to the left of the link
            return idx2 * (A(Na + i + Nx * j) - A(Na + i - 1 + Nx * j)) - idxy * (A((i - 1) + Nxa * (j + 1)) - A((i - 1) + Nxa * j)) - H * idx;
    }
    return curlcurl_link<T>(g, abei, ab, H, i, j, xdir);
}

// 2 (psi0 - psi1 U(ph)) with (s, c) = sincos(ph) (svirl/cuda/cg.h:4-12)
template <typename T> __device__ __forceinline__ C2<T> gjac_sc(C2<T> p0, T s, T c, C2<T> p1) {
    return cmk<T>(T(2) * (p0.x - (p1.x * c + p1.y * s)), T(2) * (p0.y - (p1.y * c - p1.x * s)));
}

// dF/d(Re psi) + i dF/d(Im psi) at node n (svirl/cuda/cg.h:15-121), dx*dy included.
template <typename T, typename LK>
__device__ __forceinline__ C2<T> grad_psi_node(const Geo& g, T eps0, const T* eps_sp, const C2<T>* psi, const LK& lk,
                                               int n, int i, int j, unsigned cb) {
    const T dx = GT(g, dx), dy = GT(g, dy), idx2 = GT(g, idx2), idy2 = GT(g, idy2);
    C2<T> gj = cmk<T>(T(0), T(0));
    if (cb) {
        const DuW<T> w = du_weights<T>(cb);
        const C2<T> p0 = psi[n];
        const T eps = eps_sp ? eps_sp[n] : eps0;
        const T p = p0.x * p0.x + p0.y * p0.y - eps;
        gj = cadd(gj, cscale(T(2) * w.g * p, p0));
        T sn, cs;  // the links below and left of the node enter with the opposite phase: sin(-x) = -sin(x)
        if (GL_MM(cb) || GL_MP(cb)) {
            lk.sc_sum((i - 1) + (g.Nx - 1) * j, dx, sn, cs);
            gj = cadd(gj, cscale(w.r_m0 * idx2, gjac_sc<T>(p0, -sn, cs, psi[n - 1])));
        }
        if (GL_PM(cb) || GL_PP(cb)) {
            lk.sc_sum(i + (g.Nx - 1) * j, dx, sn, cs);
            gj = cadd(gj, cscale(w.r_p0 * idx2, gjac_sc<T>(p0, sn, cs, psi[n + 1])));
        }
        if (GL_MM(cb) || GL_PM(cb)) {
            lk.sc_sum(g.Na + i + g.Nx * (j - 1), dy, sn, cs);
            gj = cadd(gj, cscale(w.r_0m * idy2, gjac_sc<T>(p0, -sn, cs, psi[n - g.Nx])));
        }
        if (GL_MP(cb) || GL_PP(cb)) {
            lk.sc_sum(g.Na + i + g.Nx * j, dy, sn, cs);
            gj = cadd(gj, cscale(w.r_0p * idy2, gjac_sc<T>(p0, sn, cs, psi[n + g.Nx])));
        }
    }
    return cscale(GT(g, dxdy), gj);
}

// dF/dA on the x link (xdir) or y link starting at node (i, j) (svirl/cuda/cg.h:124-301),
// 2*dx*dy included; exact: the boundary links use the exact derivative of the
// magnetic energy instead of the reference's doubled form.
template <typename T, typename LK>
__device__ __forceinline__ T grad_A_link(const Geo& g, T kappa2, T H, const C2<T>* psi, const T* abei, const T* ab,
                                         const LK& lk, int n, int i, int j, unsigned cb, bool xdir, bool exact = false) {
    T c = kappa2 * (exact ? curlcurl_link_exact<T>(g, abei, ab, H, i, j, xdir) : curlcurl_link<T>(g, abei, ab, H, i, j, xdir));
    if (xdir) {
        if (GL_PM(cb) || GL_PP(cb)) {
            const T r = T(0.5) * ((GL_PM(cb) ? T(1) : T(0)) + (GL_PP(cb) ? T(1) : T(0)));
            T sn, cs;
            lk.sc_sum(i + (g.Nx - 1) * j, GT(g, dx), sn, cs);
            const C2<T> p0 = psi[n], p1 = psi[n + 1];
            c += -r * GT(g, idx) * ((p0.x * p1.y - p0.y * p1.x) * cs - (p0.x * p1.x + p0.y * p1.y) * sn);
        }
    } else {
        if (GL_MP(cb) || GL_PP(cb)) {
            const T r = T(0.5) * ((GL_MP(cb) ? T(1) : T(0)) + (GL_PP(cb) ? T(1) : T(0)));
            T sn, cs;
            lk.sc_sum(g.Na + i + g.Nx * j, GT(g, dy), sn, cs);
            const C2<T> p0 = psi[n], p1 = psi[n + g.Nx];
            c += -r * GT(g, idy) * ((p0.x * p1.y - p0.y * p1.x) * cs - (p0.x * p1.x + p0.y * p1.y) * sn);
        }
    }
    return T(2) * GT(g, dxdy) * c;
}

// Line-search coefficients contributed by node n (before the dx*dy factor):
// NV = 5: c0..c4 of F(psi + a dpsi) (svirl/cuda/cg.h:314-474); NV = 17: c00..c04,
// c10..c14, c20..c24, c30, c40 of F(psi + a_psi dpsi, A + a_A dA)
// (svirl/cuda/cg.h:477-731).  dpsi(m) and dA(l) give the search direction.
// psi(m) gives the order parameter at node m, phase(l) the phase A_ei + A of link l
// (link_phase), ab5 the vector potential alone (read by the NV = 5 magnetic term
// only, which the kappa = inf callers never reach); lk the link factors of the
// node's own links.
template <typename T, int NV, typename PS, typename PH, typename FD, typename FA, typename LK>
__device__ __forceinline__ void coef_node(const Geo& g, T kappa2, T eps0, const T* eps_sp, T H, const PS& psi,
                                          const PH& phase, const T* ab5, const LK& lk, int n, int i, int j,
                                          unsigned cb, const FD& dpsi, const FA& dA, T (&c)[NV]) {
    const T dx = GT(g, dx), dy = GT(g, dy), idx = GT(g, idx), idy = GT(g, idy);
    const T idx2 = GT(g, idx2), idy2 = GT(g, idy2);
    if (cb) {
        const DuW<T> w = du_weights<T>(cb);
        const C2<T> p0 = psi(n);
        const C2<T> d0 = dpsi(n);
        const T eps = eps_sp ? eps_sp[n] : eps0;
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
            const C2<T> p1 = psi(m1), d1 = dpsi(m1);
            T s, cs;
            lk.sc_split(nl, d, s, cs);
            const C2<T> gp = grad_c_sc<T>(p0, s, cs, p1), gd = grad_c_sc<T>(d0, s, cs, d1);
            const T gg_p = gp.x * gp.x + gp.y * gp.y;
            const T gg_d = gd.x * gd.x + gd.y * gd.y;
            const T zr = gp.x * gd.x + gp.y * gd.y;  // Re(conj(gp) * gd)
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
                const C2<T> Um = cmk<T>(cs, s);  // U(-ph)
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
    if (kappa2 > T(0) && i < g.Nxc && j < g.Nyc) {
        const int Nxa = g.Nx - 1;
        const int ia00 = i + Nxa * j, ia0p = i + Nxa * (j + 1), ib00 = g.Na + i + g.Nx * j, ibp0 = g.Na + i + 1 + g.Nx * j;
        if (NV == 5) {
            const T dB = idx * (ab5[ibp0] - ab5[ib00]) - idy * (ab5[ia0p] - ab5[ia00]) - H;
            c[0] += kappa2 * dB * dB;
        } else {
            const T a00 = phase(ia00), a0p = phase(ia0p);
            const T b00 = phase(ib00), bp0 = phase(ibp0);
            const T BH = idx * (bp0 - b00) - idy * (a0p - a00) - H;
            const T dB = idx * (dA(ibp0) - dA(ib00)) - idy * (dA(ia0p) - dA(ia00));
            c[0] += kappa2 * BH * BH;
            c[1] += kappa2 * T(2) * BH * dB;
            c[2] += kappa2 * dB * dB;
        }
    }
}

}  // namespace glgpu
