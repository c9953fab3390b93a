// Batched device-side CG: every instance of a batch minimises its free energy
// with the modified nonlinear CG of svirl/solvers/cg.py (Polak-Ribiere+ beta,
// exact quartic line search in psi / quartic-in-psi, 4th-order-in-A polynomial
// for (alpha_psi, alpha_A)), with the step length, beta and the stop test decided
// on the device, so a whole CG run is one CUDA-graph launch for all instances.
//
// Per iteration: tile kernels (256 nodes of one instance per CTA) write per-tile
// FP64 partial sums; one warp per instance then adds its tiles' partials in tile
// order (deterministic) and takes the scalar decisions:
//   kb_grad -> kb_inst_beta -> kb_dir_coef -> kb_inst_alpha -> kb_update ->
//   kb_energy -> kb_inst_stop (sets the WHILE condition).
// alpha: kappa = inf, the smallest non-negative real root of dP/dalpha (the
// reference uses numpy polyroots, svirl/solvers/cg.py:227-235); finite kappa, a
// damped Newton descent of the 2-D polynomial from (0, 0) (the reference uses
// scipy BFGS from (0, 0), cg.py:378-419).  Stop: the reference's energy-ratio
// test (cg.py:315-318,541-544) or |grad F| <= gtol |grad F at the first iteration|.
// A call starts from a zero direction and beta = 0.
#include <cmath>
#include <cstring>

#include "glgpu_internal.h"
#include "glgpu_phys.cuh"

namespace glgpu {

constexpr int kPart = 17;  // doubles of per-tile partials
// The CG kernels walk tiles of kCGRep x 256 nodes of one instance: each thread
// accumulates kCGRep nodes in registers before the block reduction, so the
// reduction's cost is shared by kCGRep nodes.
constexpr int kCGRep = 4;
constexpr int kCGTile = kCGRep * kThreads;

struct CGLoop {
    int active;
    int iters;     // loop iterations done in this call
    int n_iter;
    int pad_;      // last decision of the WHILE loop (read by the host-driven loop)
    double rtol, gtol;
    int flags;     // GLGPU_CG_* bits
    int pad2_;
};

template <typename T>
__device__ __forceinline__ void store_partials(const double* v, int nv, double* out) {
    for (int k = 0; k < nv; ++k) out[k] = v[k];
}

// gradient (new buffer), Polak-Ribiere sums and |g|^2 per tile
template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_grad(const Inst* __restrict__ insts, const Tile* __restrict__ tiles, double* __restrict__ partials) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const CGState* cs = I.cg;
    if (*(volatile const int*)&cs->done) return;
    const Geo g = I.g;
    const int gi = cs->gi;
    const C2<T>* psi = (const C2<T>*)I.psi[0];
    const T* ab = (const T*)I.ab[0];
    const T* abei = (const T*)I.abei;
    C2<T>* G = (C2<T>*)I.gpsi[1 - gi];
    const C2<T>* Gp = (const C2<T>*)I.gpsi[gi];
    T* GA = (T*)I.gA[1 - gi];
    const T* GAp = (const T*)I.gA[gi];
    const TableLinks<T> lk{(const C2<T>*)I.U};
    T v[5] = {T(0), T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int r = 0; r < kCGRep; ++r) {
    const int n = t.n0 + threadIdx.x + r * kThreads;
    if (n < g.N) {
        const int i = n % g.Nx, j = n / g.Nx;
        const unsigned cb = cell_bits(g, I.mt, i, j);
        const C2<T> gv = grad_psi_node<T>(g, gsel<T>(I.epsilon, I.fepsilon), (const T*)I.eps_sp, psi, lk, n, i, j, cb);
        G[n] = gv;
        const C2<T> gp = Gp[n];
        v[0] += gv.x * (gv.x - gp.x) + gv.y * (gv.y - gp.y);
        v[1] += gp.x * gp.x + gp.y * gp.y;
        v[4] += gv.x * gv.x + gv.y * gv.y;
        if (I.solveA) {
            const T k2 = gsel<T>(I.kappa2, I.fkappa2), H = gsel<T>(I.H, I.fH);
            for (int dir = 0; dir < 2; ++dir) {
                const bool has = dir == 0 ? (i < g.Nx - 1) : (j < g.Ny - 1);
                if (!has) continue;
                const int l = dir == 0 ? i + (g.Nx - 1) * j : g.Na + i + g.Nx * j;
                const T ga = grad_A_link<T>(g, k2, H, psi, abei, ab, lk, n, i, j, cb, dir == 0, I.cg_exact != 0);
                GA[l] = ga;
                const T gap = GAp[l];
                v[2] += ga * (ga - gap);
                v[3] += gap * gap;
                v[4] += ga * ga;
            }
        }
    }
    }
    double vs[5];
    block_sum<5>(v, vs);
    if (threadIdx.x == 0) store_partials<T>(vs, 5, partials + (size_t)blockIdx.x * kPart);
}

// Sum of component k of the partials of instance I's tiles, in tile order, by one warp.
__device__ __forceinline__ double warp_tile_sum(const double* partials, int tile0, int ntiles, int k) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int q = lane; q < ntiles; q += 32) s += partials[(size_t)(tile0 + q) * kPart + k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    return __shfl_sync(0xffffffffu, s, 0);
}

// beta (Polak-Ribiere+, cg.py:422-449) and the gradient-norm stop, one warp per instance
__global__ void __launch_bounds__(128)
kb_inst_beta(const Inst* __restrict__ insts, int ninst, const double* __restrict__ partials,
                             CGLoop* loop) {
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= ninst) return;
    const Inst& I = insts[q];
    CGState* cs = I.cg;
    if (cs->done) return;
    double v[5];
    for (int k = 0; k < 5; ++k) v[k] = warp_tile_sum(partials, I.tile0, I.ntiles, k);
    if ((threadIdx.x & 31) != 0) return;
    if (cs->iter > 0) {
        cs->beta_psi = fmax(v[0] / v[1], 0.0);
        cs->beta_A = I.solveA ? fmax(v[2] / v[3], 0.0) : 0.0;
    } else {
        cs->beta_psi = 0.0;
        cs->beta_A = 0.0;
        cs->g2_0 = v[4];
    }
    cs->g2 = v[4];
    cs->gi = 1 - cs->gi;
    const bool abs_tol = (loop->flags & GLGPU_CG_GTOL_ABS) != 0;
    const double thr = abs_tol ? loop->gtol * loop->gtol : loop->gtol * loop->gtol * cs->g2_0;
    if ((cs->iter > 0 || abs_tol) && !(v[4] > thr)) {
        cs->done = 1;
        cs->status = 1;
        atomicSub(&loop->active, 1);
    }
}

// new direction (written) and the per-tile line-search coefficient partials
template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_dir_coef(const Inst* __restrict__ insts, const Tile* __restrict__ tiles, double* __restrict__ partials) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const CGState* cs = I.cg;
    if (*(volatile const int*)&cs->done) return;
    const Geo g = I.g;
    const int gi = cs->gi, di = cs->di;
    const T bp = (T)cs->beta_psi, bA = (T)cs->beta_A;
    const C2<T>* psi = (const C2<T>*)I.psi[0];
    const T* ab = (const T*)I.ab[0];
    const T* abei = (const T*)I.abei;
    const C2<T>* G = (const C2<T>*)I.gpsi[gi];
    const T* GA = (const T*)I.gA[gi];
    const C2<T>* dO = (const C2<T>*)I.dpsi[di];
    const T* dAO = (const T*)I.dA[di];
    C2<T>* dN = (C2<T>*)I.dpsi[1 - di];
    T* dAN = (T*)I.dA[1 - di];
    const TableLinks<T> lk{(const C2<T>*)I.U};
    auto dpsi = [&](int m) -> C2<T> {
        const C2<T> o = dO[m], gg = G[m];
        return cmk<T>(bp * o.x - gg.x, bp * o.y - gg.y);
    };
    auto dA = [&](int m) -> T { return bA * dAO[m] - GA[m]; };
    T c[17];
#pragma unroll
    for (int k = 0; k < 17; ++k) c[k] = T(0);
#pragma unroll 1
    for (int r = 0; r < kCGRep; ++r) {
    const int n = t.n0 + threadIdx.x + r * kThreads;
    if (n < g.N) {
        const int i = n % g.Nx, j = n / g.Nx;
        const unsigned cb = cell_bits(g, I.mt, i, j);
        dN[n] = dpsi(n);
        const T eps0 = gsel<T>(I.epsilon, I.fepsilon), H = gsel<T>(I.H, I.fH);
        if (I.solveA) {
            if (i < g.Nx - 1) { const int na = i + (g.Nx - 1) * j; dAN[na] = dA(na); }
            if (j < g.Ny - 1) { const int nb = g.Na + i + g.Nx * j; dAN[nb] = dA(nb); }
            coef_node<T, 17>(g, gsel<T>(I.kappa2, I.fkappa2), eps0, (const T*)I.eps_sp, H, psi, abei, ab, lk, n, i, j, cb,
                             dpsi, dA, c);
        } else {
            T c5[5] = {T(0), T(0), T(0), T(0), T(0)};
            coef_node<T, 5>(g, T(-1), eps0, (const T*)I.eps_sp, H, psi, abei, ab, lk, n, i, j, cb, dpsi, dA, c5);
            c[0] += c5[0]; c[5] += c5[1]; c[10] += c5[2]; c[15] += c5[3]; c[16] += c5[4];
        }
    }
    }
    double cs17[17];
    block_sum<17>(c, cs17);
    if (threadIdx.x == 0) store_partials<T>(cs17, 17, partials + (size_t)blockIdx.x * kPart);
}

// GB300 runs FP64 at a small fraction of its FP32 rate, and a single thread's
// chain of dependent FP64 operations is slow: the step lengths are found in FP32
// and then polished by FP64 Newton steps, which restore full FP64 accuracy.

// Real roots of d0 + d1 a + d2 a^2 + d3 a^3 (FP32 closed form, each root polished
// by two FP64 Newton steps on the cubic); returns the smallest root >= 0 or -1.
__device__ double smallest_nonneg_root_cubic(double d0, double d1, double d2, double d3) {
    float roots[3];
    int nr = 0;
    const double scale = fabs(d0) + fabs(d1) + fabs(d2) + fabs(d3);
    if (!(scale > 0.0)) return -1.0;
    const float f0 = (float)(d0 / scale), f1 = (float)(d1 / scale), f2 = (float)(d2 / scale), f3 = (float)(d3 / scale);
    if (fabsf(f3) <= 1e-7f) {
        if (fabsf(f2) <= 1e-7f) {
            if (f1 != 0.f) roots[nr++] = -f0 / f1;
        } else {
            const float disc = f1 * f1 - 4.f * f2 * f0;
            if (disc >= 0.f) {
                const float sq = sqrtf(disc);
                const float qq = -0.5f * (f1 + (f1 >= 0.f ? sq : -sq));
                if (qq != 0.f) roots[nr++] = f0 / qq;
                roots[nr++] = qq / f2;
            }
        }
    } else {
        const float a = f2 / f3, b = f1 / f3, c = f0 / f3;
        const float p = b - a * a / 3.f, qv = 2.f * a * a * a / 27.f - a * b / 3.f + c;
        const float disc = 0.25f * qv * qv + p * p * p / 27.f;
        if (disc > 0.f) {
            const float sq = sqrtf(disc);
            roots[nr++] = cbrtf(-0.5f * qv + sq) + cbrtf(-0.5f * qv - sq) - a / 3.f;
        } else {
            const float r = 2.f * sqrtf(-p / 3.f);
            float arg = r != 0.f ? 3.f * qv / (p * r) : 0.f;
            arg = fmaxf(-1.f, fminf(1.f, arg));
            const float phi = acosf(arg);
            for (int k = 0; k < 3; ++k) roots[nr++] = r * cosf((phi - 2.f * 3.14159265f * k) / 3.f) - a / 3.f;
        }
    }
    double best = -1.0;
    for (int k = 0; k < nr; ++k) {
        double x = (double)roots[k];
        for (int it = 0; it < 2; ++it) {  // Newton polish on the cubic, FP64
            const double f = fma(fma(fma(d3, x, d2), x, d1), x, d0), df = fma(fma(3.0 * d3, x, 2.0 * d2), x, d1);
            if (df != 0.0) x -= f / df;
        }
        if (x >= 0.0 && (best < 0.0 || x < best)) best = x;
    }
    return best;
}

// F(a, b) - c00 = sum c[i][j] a^i b^j over (i, j) != (0, 0) (17-coefficient
// layout: c00..c04, c10..c14, c20..c24, c30, c40) with its gradient and Hessian,
// by Horner's scheme: F = p0(b) + a p1(b) + a^2 p2(b) + c30 a^3 + c40 a^4 with
// quartics p_i.  The constant c00 is left out: the descent compares values of F
// that differ by far less than F itself.
template <typename T> struct P2 {
    T f, fa, fb, faa, fab, fbb;
};

template <typename T>
__device__ __forceinline__ void quartic3(const T* q, T b, T& p, T& dp, T& ddp) {
    p = fma(fma(fma(q[4], b, q[3]), b, q[2]), b, q[1]) * b + q[0];
    dp = fma(fma(fma(T(4) * q[4], b, T(3) * q[3]), b, T(2) * q[2]), b, q[1]);
    ddp = fma(fma(T(12) * q[4], b, T(6) * q[3]), b, T(2) * q[2]);
}

template <typename T>
__device__ __forceinline__ P2<T> poly2(const T (&c)[17], T a, T b) {
    T p0, p0b, p0bb, p1, p1b, p1bb, p2, p2b, p2bb;
    quartic3<T>(c + 0, b, p0, p0b, p0bb);
    quartic3<T>(c + 5, b, p1, p1b, p1bb);
    quartic3<T>(c + 10, b, p2, p2b, p2bb);
    const T c3 = c[15], c4 = c[16];
    P2<T> r;
    r.f = fma(fma(fma(fma(c4, a, c3), a, p2), a, p1), a, p0);
    r.fa = fma(fma(fma(T(4) * c4, a, T(3) * c3), a, T(2) * p2), a, p1);
    r.faa = fma(fma(T(12) * c4, a, T(6) * c3), a, T(2) * p2);
    r.fb = fma(fma(p2b, a, p1b), a, p0b);
    r.fab = fma(T(2) * p2b, a, p1b);
    r.fbb = fma(fma(p2bb, a, p1bb), a, p0bb);
    return r;
}

// Newton step of the 2-D polynomial at P (gradient steps where the Hessian is
// not positive definite).
template <typename T>
__device__ __forceinline__ void newton_dir(const P2<T>& P, T& sa, T& sb) {
    const T det = P.faa * P.fbb - P.fab * P.fab;
    if (P.faa > T(0) && det > T(0)) {
        sa = -(P.fbb * P.fa - P.fab * P.fb) / det;
        sb = -(-P.fab * P.fa + P.faa * P.fb) / det;
    } else {
        const T h = fabs(P.faa) + fabs(P.fbb) + T(1e-30);
        sa = -P.fa / h;
        sb = -P.fb / h;
    }
}

// Local minimum of the 2-D polynomial reached by a damped Newton descent from
// (0, 0) (Armijo backtracking) in FP32, then two FP64 Newton steps.  The
// polynomial is scaled to O(1) coefficients first.
__device__ bool minimise_poly2(const double (&c17)[17], double* a_out, double* b_out) {
    double scale = 0.0;
    for (int k = 1; k < 17; ++k) scale = fmax(scale, fabs(c17[k]));
    if (!(scale > 0.0)) {
        *a_out = *b_out = 0.0;
        return true;
    }
    float cf[17];
    double cd[17];
    cf[0] = 0.f;
    cd[0] = 0.0;
    for (int k = 1; k < 17; ++k) {
        cd[k] = c17[k] / scale;
        cf[k] = (float)cd[k];
    }
    float a = 0.f, b = 0.f;
    P2<float> P = poly2<float>(cf, a, b);
    const float g0 = sqrtf(P.fa * P.fa + P.fb * P.fb);
    for (int it = 0; it < 100; ++it) {
        const float gn = sqrtf(P.fa * P.fa + P.fb * P.fb);
        if (!(gn > 1e-6f * g0)) break;
        float sa, sb;
        newton_dir<float>(P, sa, sb);
        float t = 1.f;
        const float slope = P.fa * sa + P.fb * sb;
        bool moved = false;
        P2<float> Pn;
        for (int ls = 0; ls < 40; ++ls) {
            Pn = poly2<float>(cf, a + t * sa, b + t * sb);
            if (Pn.f <= P.f + 1e-4f * t * slope) {
                moved = true;
                break;
            }
            t *= 0.5f;
        }
        if (!moved) break;
        a += t * sa;
        b += t * sb;
        P = Pn;
        if (fabsf(t * sa) + fabsf(t * sb) <= 1e-7f * (1.f + fabsf(a) + fabsf(b))) break;
    }
    double ad = a, bd = b;
    for (int it = 0; it < 2; ++it) {  // FP64 polish
        const P2<double> Q = poly2<double>(cd, ad, bd);
        const double det = Q.faa * Q.fbb - Q.fab * Q.fab;
        if (!(Q.faa > 0.0 && det > 0.0)) break;
        ad += -(Q.fbb * Q.fa - Q.fab * Q.fb) / det;
        bd += -(-Q.fab * Q.fa + Q.faa * Q.fb) / det;
    }
    *a_out = ad;
    *b_out = bd;
    return isfinite(ad) && isfinite(bd);
}

// coefficients of each instance and its step lengths, one warp per instance
__global__ void __launch_bounds__(128)
kb_inst_alpha(const Inst* __restrict__ insts, int ninst, const double* __restrict__ partials,
                              CGLoop* loop) {
    const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= ninst) return;
    const Inst& I = insts[q];
    CGState* cs = I.cg;
    if (cs->done) return;
    double c[17];
#pragma unroll
    for (int k = 0; k < 17; ++k) c[k] = warp_tile_sum(partials, I.tile0, I.ntiles, k) * I.g.dxdy;
    if ((threadIdx.x & 31) != 0) return;
    bool ok;
    double ap = 0.0, aA = 0.0;
    if (I.solveA) {
        ok = minimise_poly2(c, &ap, &aA);
    } else {
        ap = smallest_nonneg_root_cubic(c[5], 2.0 * c[10], 3.0 * c[15], 4.0 * c[16]);
        ok = ap >= 0.0;
    }
    for (int k = 0; k < 17; ++k) cs->c[k] = c[k];
    cs->alpha_psi = ap;
    cs->alpha_A = aA;
    cs->di = 1 - cs->di;  // the new direction is now current
    if (!ok) {
        cs->done = 1;
        cs->status = -1;
        atomicSub(&loop->active, 1);
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_update(const Inst* __restrict__ insts, const Tile* __restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const CGState* cs = I.cg;
    if (*(volatile const int*)&cs->done) return;
    const Geo g = I.g;
    const T ap = (T)cs->alpha_psi, aA = (T)cs->alpha_A;
    C2<T>* psi = (C2<T>*)I.psi[0];
    const C2<T>* dpsi = (const C2<T>*)I.dpsi[cs->di];
    T* ab = (T*)I.ab[0];
    const T* dA = (const T*)I.dA[cs->di];
#pragma unroll
    for (int r = 0; r < kCGRep; ++r) {
        const int n = t.n0 + threadIdx.x + r * kThreads;
        if (n >= g.N) break;
        const C2<T> d = dpsi[n];
        C2<T> p = psi[n];
        p.x = ap * d.x + p.x;
        p.y = ap * d.y + p.y;
        psi[n] = p;
        if (I.solveA) {
            // new A and its link factors for the next iteration's kernels
            const int i = n % g.Nx, j = n / g.Nx;
            const T* abei = (const T*)I.abei;
            C2<T>* U = (C2<T>*)I.U;
            if (i < g.Nx - 1) {
                const int na = i + (g.Nx - 1) * j;
                const T v = aA * dA[na] + ab[na];
                ab[na] = v;
                U[na] = link_U<T>(GT(g, dx) * (abei ? abei[na] + v : v));
            }
            if (j < g.Ny - 1) {
                const int nb = g.Na + i + g.Nx * j;
                const T v = aA * dA[nb] + ab[nb];
                ab[nb] = v;
                U[nb] = link_U<T>(GT(g, dy) * (abei ? abei[nb] + v : v));
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_energy(const Inst* __restrict__ insts, const Tile* __restrict__ tiles, double* __restrict__ partials, int all) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    if (!all && *(volatile const int*)&I.cg->done) return;
    const Geo g = I.g;
    const TableLinks<T> lk{(const C2<T>*)I.U};
    T v[1] = {T(0)};
#pragma unroll
    for (int r = 0; r < kCGRep; ++r) {
        const int n = t.n0 + threadIdx.x + r * kThreads;
        if (n < g.N)
            v[0] += energy_density<T>(g, gsel<T>(I.kappa2, I.fkappa2), gsel<T>(I.epsilon, I.fepsilon),
                                      (const T*)I.eps_sp, gsel<T>(I.H, I.fH), I.mt, (const C2<T>*)I.psi[0],
                                      (const T*)I.abei, (const T*)I.ab[0], lk, n);
    }
    double vs[1];
    block_sum<1>(v, vs);
    if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kPart] = vs[0];
}

// energies, the energy-ratio stop, the iteration cap, and the WHILE condition
// (one CTA for the whole batch).
__global__ void __launch_bounds__(1024)
kb_inst_stop(const Inst* __restrict__ insts, int ninst, const double* __restrict__ partials,
                             CGLoop* loop, cudaGraphConditionalHandle cond, int use_cond) {
    const int nw = blockDim.x >> 5;
    for (int q = threadIdx.x >> 5; q < ninst; q += nw) {
        const Inst& I = insts[q];
        CGState* cs = I.cg;
        if (cs->done) continue;
        const double E = warp_tile_sum(partials, I.tile0, I.ntiles, 0) * I.g.dxdy;
        if ((threadIdx.x & 31) != 0) continue;
        cs->E_prev = cs->E;
        cs->E = E;
        const int it = cs->iter;
        cs->iter = it + 1;
        if (it > 0 && fabs(E / cs->E_prev - 1.0) < loop->rtol) {
            cs->done = 1;
            cs->status = 2;
            atomicSub(&loop->active, 1);
        } else if (I.cg_target == I.cg_target && E <= I.cg_target + I.cg_target_tol * fabs(I.cg_target)) {
            cs->done = 1;
            cs->status = 4;
            atomicSub(&loop->active, 1);
        } else if (cs->iter >= loop->n_iter) {
            cs->done = 1;
            cs->status = 3;
            atomicSub(&loop->active, 1);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const int iters = loop->iters + 1;
        loop->iters = iters;
        const int act = atomicAdd(&loop->active, 0);
        const unsigned go = (act > 0 && iters < loop->n_iter + 2) ? 1u : 0u;
        if (use_cond) cudaGraphSetConditional(cond, go);
        loop->pad_ = (int)go;
    }
}

// start of a CG call: zero direction and gradient, the link-factor table of the
// start state (TableLinks), then the energy of the start state
template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_zero_dir(const Inst* __restrict__ insts, const Tile* __restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const Geo g = I.g;
#pragma unroll
    for (int r = 0; r < kCGRep; ++r) {
        const int n = t.n0 + threadIdx.x + r * kThreads;
        if (n >= g.N) break;
        ((C2<T>*)I.dpsi[0])[n] = cmk<T>(T(0), T(0));
        ((C2<T>*)I.gpsi[0])[n] = cmk<T>(T(0), T(0));
        const int i = n % g.Nx, j = n / g.Nx;
        const T* abei = (const T*)I.abei;
        const T* ab = (const T*)I.ab[0];
        C2<T>* U = (C2<T>*)I.U;
        if (i < g.Nx - 1) {
            const int na = i + (g.Nx - 1) * j;
            ((T*)I.dA[0])[na] = T(0);
            ((T*)I.gA[0])[na] = T(0);
            U[na] = link_U<T>(GT(g, dx) * link_phase(abei, ab, na));
        }
        if (j < g.Ny - 1) {
            const int nb = g.Na + i + g.Nx * j;
            ((T*)I.dA[0])[nb] = T(0);
            ((T*)I.gA[0])[nb] = T(0);
            U[nb] = link_U<T>(GT(g, dy) * link_phase(abei, ab, nb));
        }
    }
}

__global__ void __launch_bounds__(1024)
kb_init(const Inst* __restrict__ insts, int ninst, const double* __restrict__ partials, CGLoop* loop,
                        cudaGraphConditionalHandle cond, int use_cond) {
    const int nw = blockDim.x >> 5;
    for (int q = threadIdx.x >> 5; q < ninst; q += nw) {
        const Inst& I = insts[q];
        const double E = warp_tile_sum(partials, I.tile0, I.ntiles, 0) * I.g.dxdy;
        if ((threadIdx.x & 31) != 0) continue;
        CGState* cs = I.cg;
        cs->beta_psi = cs->beta_A = 0.0;
        cs->alpha_psi = cs->alpha_A = 0.0;
        cs->E = E;
        cs->E_prev = E;
        cs->g2 = cs->g2_0 = 0.0;
        cs->iter = 0;
        cs->done = 0;
        cs->gi = 0;
        cs->di = 0;
        cs->status = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        loop->active = ninst;
        loop->iters = 0;
        const unsigned go = (ninst > 0 && loop->n_iter > 0) ? 1u : 0u;
        if (use_cond) cudaGraphSetConditional(cond, go);
        loop->pad_ = (int)go;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct CGLaunch {
    const Inst* insts;
    const Tile* tiles;
    double* partials;
    CGLoop* loop;
    int ninst, ntiles, dtype;
};

static void* fn_grad(int dt) { return dt == 8 ? (void*)kb_grad<double> : (void*)kb_grad<float>; }
static void* fn_dir_coef(int dt) { return dt == 8 ? (void*)kb_dir_coef<double> : (void*)kb_dir_coef<float>; }
static void* fn_update(int dt) { return dt == 8 ? (void*)kb_update<double> : (void*)kb_update<float>; }
static void* fn_energy(int dt) { return dt == 8 ? (void*)kb_energy<double> : (void*)kb_energy<float>; }
static void* fn_zero_dir(int dt) { return dt == 8 ? (void*)kb_zero_dir<double> : (void*)kb_zero_dir<float>; }

static inline int warp_blocks(int ninst) { return (ninst + 3) / 4; }  // 4 warps of 32 per CTA

// Host-driven loop body (the graph holds the same launches).
static cudaError_t cg_launch_body(const CGLaunch& L, cudaStream_t s) {
    const cudaGraphConditionalHandle none = 0;
    const int wb = warp_blocks(L.ninst);
    if (L.dtype == 8) kb_grad<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials);
    else kb_grad<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials);
    kb_inst_beta<<<wb, 128, 0, s>>>(L.insts, L.ninst, L.partials, L.loop);
    if (L.dtype == 8) kb_dir_coef<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials);
    else kb_dir_coef<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials);
    kb_inst_alpha<<<wb, 128, 0, s>>>(L.insts, L.ninst, L.partials, L.loop);
    if (L.dtype == 8) kb_update<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
    else kb_update<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
    if (L.dtype == 8) kb_energy<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials, 0);
    else kb_energy<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials, 0);
    kb_inst_stop<<<1, 1024, 0, s>>>(L.insts, L.ninst, L.partials, L.loop, none, 0);
    return cudaGetLastError();
}

static cudaError_t cg_launch_prologue(const CGLaunch& L, cudaStream_t s) {
    const cudaGraphConditionalHandle none = 0;
    if (L.dtype == 8) kb_zero_dir<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
    else kb_zero_dir<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
    if (L.dtype == 8) kb_energy<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials, 1);
    else kb_energy<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.partials, 1);
    kb_init<<<1, 1024, 0, s>>>(L.insts, L.ninst, L.partials, L.loop, none, 0);
    return cudaGetLastError();
}

#define GCHK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { err = e_; goto fail; } } while (0)

// The whole CG run of all instances as one graph:
//   zero_dir -> energy -> init -> WHILE(active) {
//       grad -> beta -> dir_coef -> alpha -> update -> energy -> stop }
static cudaError_t build_cg_graph(const CGLaunch& L, cudaGraphExec_t* exec) {
    cudaError_t err = cudaSuccess;
    cudaGraph_t top = nullptr, body = nullptr;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t prev = nullptr, nd;
    int zero = 0, one = 1;
    const dim3 gt(L.ntiles), bt(kThreads), gw(warp_blocks(L.ninst)), bw(128), g1(1), b1(1024);
    const Inst* insts = L.insts;
    const Tile* tiles = L.tiles;
    double* partials = L.partials;
    CGLoop* loop = L.loop;
    int ninst = L.ninst;

    GCHK(cudaGraphCreate(&top, 0));
    GCHK(cudaGraphConditionalHandleCreate(&h, top, 0, cudaGraphCondAssignDefault));
    {
        void* a[] = {&insts, &tiles};
        GCHK(add_kernel(top, &nd, nullptr, 0, fn_zero_dir(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &tiles, &partials, &one};
        GCHK(add_kernel(top, &nd, &prev, 1, fn_energy(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &ninst, &partials, &loop, &h, &one};
        GCHK(add_kernel(top, &nd, &prev, 1, (void*)kb_init, g1, b1, a));
        prev = nd;
    }
    GCHK(add_while(top, &nd, &prev, 1, h, &body));
    prev = nullptr;
    {
        void* a[] = {&insts, &tiles, &partials};
        GCHK(add_kernel(body, &nd, nullptr, 0, fn_grad(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &ninst, &partials, &loop};
        GCHK(add_kernel(body, &nd, &prev, 1, (void*)kb_inst_beta, gw, bw, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &tiles, &partials};
        GCHK(add_kernel(body, &nd, &prev, 1, fn_dir_coef(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &ninst, &partials, &loop};
        GCHK(add_kernel(body, &nd, &prev, 1, (void*)kb_inst_alpha, gw, bw, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &tiles};
        GCHK(add_kernel(body, &nd, &prev, 1, fn_update(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &tiles, &partials, &zero};
        GCHK(add_kernel(body, &nd, &prev, 1, fn_energy(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &ninst, &partials, &loop, &h, &one};
        GCHK(add_kernel(body, &nd, &prev, 1, (void*)kb_inst_stop, g1, b1, a));
    }
    GCHK(cudaGraphInstantiate(exec, top, 0));
    cudaGraphDestroy(top);
    return cudaSuccess;
fail:
    if (top) cudaGraphDestroy(top);
    *exec = nullptr;
    return err;
}
#undef GCHK

int batch_set_energy_targets(glgpu_batch* b, const double* targets, double rel_tol) {
    if (!targets) {
        b->cg_targets.clear();
        return GLGPU_OK;
    }
    if (!(rel_tol >= 0.0)) return batch_error(b, GLGPU_E_ARG, "batch_set_energy_targets: rel_tol < 0");
    b->cg_targets.assign(targets, targets + b->ninst);
    b->cg_target_tol = rel_tol;
    return GLGPU_OK;
}

int batch_cg(glgpu_batch* b, int n_iter, double rtol, double gtol, int flags, int32_t* iters, double* energies, double* grad_rel,
             int32_t* status, double* elapsed_ms) {
    if (n_iter < 0 || !(rtol >= 0.0) || !(gtol >= 0.0)) return batch_error(b, GLGPU_E_ARG, "batch_cg: bad n_iter, rtol or gtol");
    std::vector<Inst> insts(b->ninst);
    std::vector<Tile> cgtiles;
    for (int q = 0; q < b->ninst; ++q) {
        glgpu_handle* h = b->hs[q];
        const int rc = cg_ensure(h);
        if (rc) return batch_error(b, rc, "batch_cg: " + h->last_error);
        cudaStreamSynchronize(h->stream);
        insts[q] = h->inst_h;
        // this copy of the descriptors indexes the CG tile table (kCGTile nodes per tile)
        insts[q].tile0 = (int)cgtiles.size();
        for (int n0 = 0; n0 < h->g.N; n0 += kCGTile) cgtiles.push_back(Tile{q, n0});
        insts[q].ntiles = (int)cgtiles.size() - insts[q].tile0;
        insts[q].cg_exact = (flags & GLGPU_CG_EXACT_BOUNDARY) ? 1 : 0;
        insts[q].cg_target = b->cg_targets.empty() ? NAN : b->cg_targets[q];
        insts[q].cg_target_tol = b->cg_target_tol;
    }
    if (!b->cg_tiles) {
        b->cg_ntiles = (int)cgtiles.size();
        if (cudaMalloc(&b->cg_tiles, sizeof(Tile) * cgtiles.size()) != cudaSuccess ||
            cudaMemcpy(b->cg_tiles, cgtiles.data(), sizeof(Tile) * cgtiles.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return batch_error(b, GLGPU_E_OOM, "batch_cg: cannot place the tile table");
    }
    if (!b->cg_partials && cudaMalloc(&b->cg_partials, sizeof(double) * kPart * (size_t)b->cg_ntiles) != cudaSuccess)
        return batch_error(b, GLGPU_E_OOM, "batch_cg: out of device memory");
    if (!b->cg_loop && cudaMalloc(&b->cg_loop, sizeof(CGLoop)) != cudaSuccess)
        return batch_error(b, GLGPU_E_OOM, "batch_cg: out of device memory");
    cudaStream_t s = b->stream;
    CGLoop lp;
    memset(&lp, 0, sizeof(lp));
    lp.n_iter = n_iter;
    lp.rtol = rtol;
    lp.gtol = gtol;
    lp.flags = flags;
    cudaError_t e = cudaMemcpyAsync(b->insts, insts.data(), sizeof(Inst) * insts.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->cg_loop, &lp, sizeof(lp), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return batch_error(b, GLGPU_E_CUDA, std::string("batch_cg: ") + cudaGetErrorString(e));
    CGLaunch L;
    L.insts = b->insts;
    L.tiles = (const Tile*)b->cg_tiles;
    L.partials = b->cg_partials;
    L.loop = (CGLoop*)b->cg_loop;
    L.ninst = b->ninst;
    L.ntiles = b->cg_ntiles;
    L.dtype = b->dtype;
    if (b->use_graphs && !b->cg_graph_failed && !b->cg_exec && build_cg_graph(L, &b->cg_exec) != cudaSuccess) {
        b->cg_graph_failed = true;
        cudaGetLastError();
    }
    const bool graph = b->use_graphs && b->cg_exec != nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (elapsed_ms) {
        cudaEventCreate(&ev0);
        cudaEventCreate(&ev1);
        cudaEventRecord(ev0, s);
    }
    if (graph) {
        e = cudaGraphLaunch(b->cg_exec, s);
    } else {
        e = cg_launch_prologue(L, s);
        int* go_h = nullptr;
        if (e == cudaSuccess) e = cudaMallocHost(&go_h, sizeof(int));
        for (int it = 0; e == cudaSuccess && it < n_iter + 1; ++it) {
            *go_h = 0;
            e = cudaMemcpyAsync(go_h, &L.loop->pad_, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess || !*go_h) break;
            e = cg_launch_body(L, s);
        }
        if (go_h) cudaFreeHost(go_h);
    }
    if (elapsed_ms) cudaEventRecord(ev1, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (elapsed_ms) {
        float ms = 0.f;
        if (e == cudaSuccess) cudaEventElapsedTime(&ms, ev0, ev1);
        *elapsed_ms = ms;
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
    }
    if (e != cudaSuccess) return batch_error(b, GLGPU_E_CUDA, std::string("batch_cg: ") + cudaGetErrorString(e));
    int nfail = 0;
    for (int q = 0; q < b->ninst; ++q) {
        CGState cs;
        e = cudaMemcpy(&cs, b->hs[q]->cgst, sizeof(cs), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return batch_error(b, GLGPU_E_CUDA, std::string("batch_cg: ") + cudaGetErrorString(e));
        if (iters) iters[q] = cs.iter;
        if (energies) energies[q] = cs.E;
        if (grad_rel) grad_rel[q] = cs.g2_0 > 0.0 ? std::sqrt(cs.g2 / cs.g2_0) : 0.0;
        if (status) status[q] = cs.status;
        if (cs.status < 0) ++nfail;
    }
    if (nfail)
        return batch_error(b, GLGPU_E_NOROOT, "batch_cg: no descent step for " + std::to_string(nfail) + " instance(s)");
    return GLGPU_OK;
}

}  // namespace glgpu
