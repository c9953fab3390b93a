// Batched device-side CG: every instance of a batch minimises its free energy
// with the modified nonlinear CG of svirl/solvers/cg.py (Polak-Ribiere+ beta,
// exact quartic line search in psi / quartic-in-psi, 4th-order-in-A polynomial
// for (alpha_psi, alpha_A)), with the step length, beta and the stop test decided
// on the device, so a whole CG run is one CUDA-graph launch for all instances.
//
// Per iteration three tile kernels (rep x 256 nodes of one instance per CTA) write
// per-tile FP64 partial sums; in each, the CTA that finishes an instance's last
// tile adds that instance's partials in tile order (one warp, deterministic) and
// takes the instance's scalar decisions:
//   kb_grad (+ beta, gradient stop) -> kb_dir_coef (+ step lengths) ->
//   kb_step (update, energy, + energy stop; the launch's last CTA sets the WHILE
//   condition).
// The state alternates between buffers 0 and 1 (psi[pi], ab[pi]) so that kb_step
// reads the old state while it writes the new one; kb_finish copies it back to
// buffer 0 at the end of a call.
// alpha: kappa = inf, the smallest non-negative real root of dP/dalpha (the
// reference uses numpy polyroots, svirl/solvers/cg.py:227-235); finite kappa, a
// damped Newton descent of the 2-D polynomial from (0, 0) (the reference uses
// scipy BFGS from (0, 0), cg.py:378-419).  Stop: the reference's energy-ratio
// test (cg.py:315-318,541-544) or |grad F| <= gtol |grad F at the first iteration|.
// A call starts from a zero direction and beta = 0.
#include <cmath>
#include <cstring>
#include <type_traits>

#include "glgpu_internal.h"
#include "glgpu_phys.cuh"

namespace glgpu {

constexpr int kPart = 17;  // doubles of per-tile partials
// The CG kernels walk tiles of rep x 256 nodes of one instance: each thread
// accumulates rep nodes in registers before the block reduction, so the
// reduction's cost is shared by rep nodes.  rep (2, 4 or 8) is a property of the
// instance alone (cg_rep_of), so an instance's arithmetic, and with it its CG
// run, does not depend on the batch it is in.
constexpr int kCGRepMax = 8;
struct CGTile {
    int inst, n0, rep, pad;
};

// Tile depth of an instance of N nodes: the deepest of 8, 4, 2 that still cuts
// it into at least kCGMinTiles tiles (so that an instance run alone spreads over
// a quarter of the SMs), else 2.  Deeper tiles share each block reduction among
// more nodes: 64 instances, 7.19M nodes: 0.77 ms per iteration with depth 4 for
// all, 0.70 with 8 for all.
constexpr int kCGMinTiles = 38;
static int cg_rep_of(int N) {
    for (int r = kCGRepMax; r > 2; r /= 2)
        if ((N + kThreads * r - 1) / (kThreads * r) >= kCGMinTiles) return r;
    return 2;
}
// Resident CTAs per SM asked of the compiler for the FP32 CG kernels (caps their
// registers at 65536 / (kThreads * minimum CTAs)), per kernel.  Measured on the
// 64-instance field sweep (ms per iteration, grad / coef / step caps; one box):
// 5/4/4 0.694, 4/4/4 0.702 (the step kernel fits 64 registers without spilling),
// 6/4/4 0.702, 5/3/4 0.710, 4/4/1 0.715; on another box 4/4/1 0.708, 5/4/1 0.701,
// 4/4/3 0.715, 5/5/1 0.724; earlier 6/6, 8/4, 4/8 and 8/8 0.79-1.09, 3/3 and 2/2
// 0.82-0.94.
#ifndef GLGPU_CG_MINB
#define GLGPU_CG_MINB 4
#endif
#ifndef GLGPU_CG_MINB_GRAD
#define GLGPU_CG_MINB_GRAD 5
#endif
#ifndef GLGPU_CG_MINB_COEF
#define GLGPU_CG_MINB_COEF GLGPU_CG_MINB
#endif
// nodes of a tile whose line-search terms one thread computes together (1: one
// node at a time)
#ifndef GLGPU_CG_COEF_UNROLL
#define GLGPU_CG_COEF_UNROLL 1
#endif
constexpr int kCoefUnroll = GLGPU_CG_COEF_UNROLL;

struct CGLoop {
    int active;
    int iters;     // loop iterations done in this call
    int n_iter;
    int pad_;      // last decision of the WHILE loop (read by the host-driven loop)
    double rtol, gtol;
    int flags;     // GLGPU_CG_* bits
    int ticket;    // CTAs finished in the running launch of the step kernel
    int window;    // energy-window stop: every `window` iterations (0: off) ...
    int pad2_;
    double wtol;   // ... stop unless E fell by more than wtol |E| since the last mark
};

template <typename T>
__device__ __forceinline__ void store_partials(const double* v, int nv, double* out) {
    for (int k = 0; k < nv; ++k) out[k] = v[k];
}

// Components 0..NV-1 of the partials of one instance's tiles summed by one
// warp (lane l adds tiles l, l+32, ... in order, then a fixed shuffle tree),
// every lane receiving the sums.  All NV components are loaded per tile, so the
// loads and the shuffle levels of the components overlap.
template <int NV>
__device__ __forceinline__ void warp_tile_sums(const double* partials, int tile0, int ntiles, double (&s)[NV]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] = 0.0;
#pragma unroll 4
    for (int q = lane; q < ntiles; q += 32) {
        const double* p = partials + (size_t)(tile0 + q) * kPart;
        double t[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) t[k] = __ldcg(p + k);  // written by other CTAs of this launch
#pragma unroll
        for (int k = 0; k < NV; ++k) s[k] += t[k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < NV; ++k) s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] = __shfl_sync(0xffffffffu, s[k], 0);
}

// The same sums by a whole CTA, times `scale`, into out[] (shared memory): warp w
// adds components w, w + kWarps, ..., each exactly as warp_tile_sums does, so
// the FP64 additions are spread over the CTA's warps.  Ends with a barrier.
template <int NV>
__device__ __forceinline__ void cta_tile_sums(const double* partials, int tile0, int ntiles, double scale,
                                              double* out) {
    constexpr int KPW = (NV + kWarps - 1) / kWarps;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double s[KPW];
#pragma unroll
    for (int c = 0; c < KPW; ++c) s[c] = 0.0;
    for (int q = lane; q < ntiles; q += 32) {
        const double* p = partials + (size_t)(tile0 + q) * kPart;
#pragma unroll
        for (int c = 0; c < KPW; ++c)
            if (w + c * kWarps < NV) s[c] += __ldcg(p + w + c * kWarps);  // written by other CTAs of this launch
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < KPW; ++c) s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < KPW; ++c)
            if (w + c * kWarps < NV) out[w + c * kWarps] = s[c] * scale;
    __syncthreads();
}

// beta (Polak-Ribiere+, cg.py:422-449) and the gradient-norm stop of one
// instance, by the CTA that finished its last tile
__device__ __noinline__ void inst_beta(const Inst& I, CGState* cs, const double* partials, CGLoop* loop) {
    __shared__ double v[5];
    cta_tile_sums<5>(partials, I.tile0, I.ntiles, 1.0, v);
    if (threadIdx.x != 0) return;
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

// The CTA that finishes the last tile of an instance in a launch (a ticket per
// instance) takes that instance's scalar decisions: the instance's partials are
// then all stored.  The ticket is left at 0 for the next launch.
__device__ __forceinline__ bool last_cta_of_instance(CGState* cs, int ntiles) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        __threadfence();
        const int tk = atomicAdd(&cs->ticket, 1);
        s_last = tk == ntiles - 1;
        if (s_last) cs->ticket = 0;
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last;
}

// The tile bodies take every field as a __restrict__ pointer (the buffers are
// distinct), so the compiler may keep loaded values across the stores, and they
// store a node's results after its loads.

// Prefetch (to L2) of what the gradient of node n reads, issued GLGPU_CG_PREFETCH
// nodes of the tile ahead (0: off) so that a node's loads find their lines on
// chip: the node's psi row neighbourhood, its link factors and cell bits, its
// previous gradient and the vector potential of the links around it.  No effect on
// the results.  At the first node of a tile the next GLGPU_CG_PREFETCH nodes are
// prefetched together.
#ifndef GLGPU_CG_PREFETCH
#define GLGPU_CG_PREFETCH 1
#endif
constexpr int kCGPrefetch = GLGPU_CG_PREFETCH;
// calls pf(q) for the tile positions to prefetch at position r of a tile of rep
template <typename PF> __device__ __forceinline__ void cg_prefetch_ahead(int r, int rep, const PF& pf) {
    if (kCGPrefetch <= 0) return;
    if (r == 0) {
#pragma unroll
        for (int q = 1; q <= kCGPrefetch; ++q)
            if (q < rep) pf(q);
    } else if (r + kCGPrefetch < rep) {
        pf(r + kCGPrefetch);
    }
}
__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
template <typename T>
__device__ __forceinline__ void grad_prefetch(const Inst& I, const Geo& g, int n, const C2<T>* psi, const C2<T>* U,
                                              const C2<T>* Gp, const T* ab, const T* GAp) {
    if (n >= g.N) return;
    const int i = n % g.Nx, j = n / g.Nx;
    prefetch_l2(I.cbits + n);
    prefetch_l2(psi + n);
    if (j > 0) prefetch_l2(psi + n - g.Nx);
    if (j + 1 < g.Ny) prefetch_l2(psi + n + g.Nx);
    prefetch_l2(Gp + n);
    const int la = i + (g.Nx - 1) * j, lb = g.Na + i + g.Nx * j;
    if (i + 1 < g.Nx) prefetch_l2(U + la);
    if (j + 1 < g.Ny) prefetch_l2(U + lb);
    if (j > 0) prefetch_l2(U + lb - g.Nx);
    if (I.solveA && ab) {
        if (i + 1 < g.Nx) {
            prefetch_l2(ab + la);
            prefetch_l2(GAp + la);
            if (j > 0) prefetch_l2(ab + la - (g.Nx - 1));
            if (j + 1 < g.Ny) prefetch_l2(ab + la + (g.Nx - 1));
        }
        if (j + 1 < g.Ny) {
            prefetch_l2(ab + lb);
            prefetch_l2(GAp + lb);
        }
        if (j > 0) prefetch_l2(ab + lb - g.Nx);
    }
}

// The same one node ahead for the direction / line-search kernel (state, previous
// direction and new gradient at the node and its +x / +y neighbours, links) and
// for the step kernel (state and direction at the node and its +y neighbour,
// links of the node's cell).
template <typename T>
__device__ __forceinline__ void coef_prefetch(const Inst& I, const Geo& g, int n, const C2<T>* psi, const C2<T>* U,
                                              const C2<T>* G, const C2<T>* dO, const T* ab, const T* GA,
                                              const T* dAO) {
    if (n >= g.N) return;
    const int i = n % g.Nx, j = n / g.Nx;
    prefetch_l2(I.cbits + n);
    prefetch_l2(psi + n);
    prefetch_l2(G + n);
    prefetch_l2(dO + n);
    if (j + 1 < g.Ny) {
        prefetch_l2(psi + n + g.Nx);
        prefetch_l2(G + n + g.Nx);
        prefetch_l2(dO + n + g.Nx);
    }
    const int la = i + (g.Nx - 1) * j, lb = g.Na + i + g.Nx * j;
    if (i + 1 < g.Nx) prefetch_l2(U + la);
    if (j + 1 < g.Ny) prefetch_l2(U + lb);
    if (I.solveA && ab) {
        if (i + 1 < g.Nx) {
            prefetch_l2(ab + la);
            prefetch_l2(GA + la);
            prefetch_l2(dAO + la);
            if (j + 1 < g.Ny) {
                prefetch_l2(ab + la + (g.Nx - 1));
                prefetch_l2(GA + la + (g.Nx - 1));
                prefetch_l2(dAO + la + (g.Nx - 1));
            }
        }
        if (j + 1 < g.Ny) {
            prefetch_l2(ab + lb);
            prefetch_l2(GA + lb);
            prefetch_l2(dAO + lb);
        }
    }
}
template <typename T>
__device__ __forceinline__ void step_prefetch(const Inst& I, const Geo& g, int n, const C2<T>* psi, const C2<T>* dpsi,
                                              const T* ab, const T* dA) {
    if (n >= g.N) return;
    const int i = n % g.Nx, j = n / g.Nx;
    prefetch_l2(I.cbits + n);
    prefetch_l2(psi + n);
    prefetch_l2(dpsi + n);
    if (j + 1 < g.Ny) {
        prefetch_l2(psi + n + g.Nx);
        prefetch_l2(dpsi + n + g.Nx);
    }
    if (I.solveA && ab) {
        const int la = i + (g.Nx - 1) * j, lb = g.Na + i + g.Nx * j;
        if (i + 1 < g.Nx) {
            prefetch_l2(ab + la);
            prefetch_l2(dA + la);
            if (j + 1 < g.Ny) {
                prefetch_l2(ab + la + (g.Nx - 1));
                prefetch_l2(dA + la + (g.Nx - 1));
            }
        }
        if (j + 1 < g.Ny) {
            prefetch_l2(ab + lb);
            prefetch_l2(dA + lb);
        }
    }
}

// gradient (new buffer), Polak-Ribiere sums and |g|^2 of one tile
template <typename T, bool SA>
__device__ __forceinline__ void grad_tile(const Inst& I, int n0, int rep, const C2<T>* __restrict__ psi,
                                          const T* __restrict__ ab, const T* __restrict__ abei,
                                          const C2<T>* __restrict__ U, C2<T>* __restrict__ G,
                                          const C2<T>* __restrict__ Gp, T* __restrict__ GA,
                                          const T* __restrict__ GAp, T (&v)[5]) {
    const Geo g = I.g;
    const TableLinks<T> lk{U};
    const T eps0 = gsel<T>(I.epsilon, I.fepsilon), k2 = gsel<T>(I.kappa2, I.fkappa2), H = gsel<T>(I.H, I.fH);
#pragma unroll
    for (int r = 0; r < kCGRepMax; ++r) {
        if (r >= rep) break;
        const int n = n0 + threadIdx.x + r * kThreads;
        cg_prefetch_ahead(r, rep, [&](int q) { grad_prefetch<T>(I, g, n0 + threadIdx.x + q * kThreads, psi, U, Gp, ab, GAp); });
        if (n < g.N) {
            const int i = n % g.Nx, j = n / g.Nx;
            const unsigned cb = I.cbits[n];
            const C2<T> gv = grad_psi_node<T>(g, eps0, (const T*)I.eps_sp, psi, lk, n, i, j, cb);
            const C2<T> gp = Gp[n];
            v[0] += gv.x * (gv.x - gp.x) + gv.y * (gv.y - gp.y);
            v[1] += gp.x * gp.x + gp.y * gp.y;
            v[4] += gv.x * gv.x + gv.y * gv.y;
            T ga[2] = {T(0), T(0)};
            const bool has[2] = {i < g.Nx - 1, j < g.Ny - 1};
            const int l[2] = {i + (g.Nx - 1) * j, g.Na + i + g.Nx * j};
            if (SA) {
#pragma unroll
                for (int dir = 0; dir < 2; ++dir) {
                    if (!has[dir]) continue;
                    ga[dir] = grad_A_link<T>(g, k2, H, psi, abei, ab, lk, n, i, j, cb, dir == 0, I.cg_exact != 0);
                    const T gap = GAp[l[dir]];
                    v[2] += ga[dir] * (ga[dir] - gap);
                    v[3] += gap * gap;
                    v[4] += ga[dir] * ga[dir];
                }
            }
            G[n] = gv;
            if (SA)
#pragma unroll
                for (int dir = 0; dir < 2; ++dir)
                    if (has[dir]) GA[l[dir]] = ga[dir];
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? GLGPU_CG_MINB_GRAD : 1)
kb_grad(const Inst* __restrict__ insts, const CGTile* __restrict__ tiles, double* __restrict__ partials, CGLoop* loop) {
    const CGTile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    CGState* cs = I.cg;
    if (*(volatile const int*)&cs->done) return;
    const int gi = cs->gi, pi = cs->pi;
    T v[5] = {T(0), T(0), T(0), T(0), T(0)};
    auto run = [&](auto sa) {
        grad_tile<T, decltype(sa)::value>(I, t.n0, t.rep, (const C2<T>*)I.psi[pi], (const T*)I.ab[I.solveA ? pi : 0],
                                          (const T*)I.abei, (const C2<T>*)I.U, (C2<T>*)I.gpsi[1 - gi],
                                          (const C2<T>*)I.gpsi[gi], (T*)I.gA[1 - gi], (const T*)I.gA[gi], v);
    };
    if (I.solveA) run(std::true_type{});
    else run(std::false_type{});
    double vs[5];
    block_sum<5>(v, vs);
    if (threadIdx.x == 0) store_partials<T>(vs, 5, partials + (size_t)blockIdx.x * kPart);
    if (last_cta_of_instance(cs, I.ntiles)) inst_beta(I, cs, partials, loop);
}

// GB300 runs FP64 at a small fraction of its FP32 rate, and a single thread's
// chain of dependent FP64 operations is slow: the step lengths are found in FP32
// and, for FP64 instances, polished by FP64 Newton steps, which restore full FP64
// accuracy (FP32 instances polish in FP32).

// Real roots of d0 + d1 a + d2 a^2 + d3 a^3 (FP32 closed form, each root polished
// by two Newton steps on the cubic, in FP64 when FP64); returns the smallest
// root >= 0 or -1.
template <bool FP64>
__device__ double smallest_nonneg_root_cubic(double d0, double d1, double d2, double d3) {
    float roots[3];
    int nr = 0;
    const double scale = fabs(d0) + fabs(d1) + fabs(d2) + fabs(d3);
    if (!(scale > 0.0)) return -1.0;
    int e;
    frexp(scale, &e);
    const double inv = ldexp(1.0, -e);  // power of two: the scaling is exact
    const float f0 = (float)(d0 * inv), f1 = (float)(d1 * inv), f2 = (float)(d2 * inv), f3 = (float)(d3 * inv);
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
        double x;
        if (FP64) {
            x = (double)roots[k];
            for (int it = 0; it < 2; ++it) {  // Newton polish on the cubic, FP64
                const double f = fma(fma(fma(d3, x, d2), x, d1), x, d0), df = fma(fma(3.0 * d3, x, 2.0 * d2), x, d1);
                if (df != 0.0) x -= f / df;
            }
        } else {
            float xf = roots[k];
            for (int it = 0; it < 2; ++it) {  // Newton polish on the scaled cubic, FP32
                const float f = fmaf(fmaf(fmaf(f3, xf, f2), xf, f1), xf, f0);
                const float df = fmaf(fmaf(3.f * f3, xf, 2.f * f2), xf, f1);
                if (df != 0.f) xf -= f / df;
            }
            x = (double)xf;
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
// (0, 0) (Armijo backtracking) in FP32, then, when FP64, two FP64 Newton steps.
// cf / cd: the coefficients scaled to O(1) (c00 = 0), in FP32 / FP64.
template <bool FP64>
__device__ bool minimise_poly2(const float* cfs, const double* cds, double* a_out, double* b_out) {
    float cf[17];
#pragma unroll
    for (int k = 0; k < 17; ++k) cf[k] = cfs[k];
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
    if constexpr (FP64) {
        double cd[17];
#pragma unroll
        for (int k = 0; k < 17; ++k) cd[k] = cds[k];
        for (int it = 0; it < 2; ++it) {  // FP64 polish
            const P2<double> Q = poly2<double>(cd, ad, bd);
            const double det = Q.faa * Q.fbb - Q.fab * Q.fab;
            if (!(Q.faa > 0.0 && det > 0.0)) break;
            const double idet = 1.0 / det;
            ad -= (Q.fbb * Q.fa - Q.fab * Q.fb) * idet;
            bd -= (Q.faa * Q.fb - Q.fab * Q.fa) * idet;
        }
    }
    *a_out = ad;
    *b_out = bd;
    return isfinite(ad) && isfinite(bd);
}

// line-search coefficients of one instance and its step lengths, by the CTA
// that finished its last tile (the sums on all warps, the scaling on warp 0,
// the search on thread 0)
template <bool FP64>
__device__ __noinline__ void inst_alpha(const Inst& I, CGState* cs, const double* partials, CGLoop* loop) {
    __shared__ double c[17], cd[17];
    __shared__ float cf[17];
    cta_tile_sums<17>(partials, I.tile0, I.ntiles, I.g.dxdy, c);
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    bool ok = true;
    double ap = 0.0, aA = 0.0;
    if (I.solveA) {
        // scale: the largest |c_k| (k >= 1) as a power of two, so the scaling is exact
        double m = (lane >= 1 && lane < 17) ? fabs(c[lane]) : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (m > 0.0) {
            int e;
            frexp(m, &e);
            const double inv = ldexp(1.0, -e);
            if (lane < 17) {
                const double d = lane == 0 ? 0.0 : c[lane] * inv;
                cd[lane] = d;
                cf[lane] = (float)d;
            }
            __syncwarp();
            if (lane == 0) ok = minimise_poly2<FP64>(cf, cd, &ap, &aA);
        }
    } else if (lane == 0) {
        ap = smallest_nonneg_root_cubic<FP64>(c[5], 2.0 * c[10], 3.0 * c[15], 4.0 * c[16]);
        ok = ap >= 0.0;
    }
    if (lane != 0) return;
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

// new direction (written) and the line-search coefficients of one tile
template <typename T, bool SA>
__device__ __forceinline__ void dir_coef_tile(const Inst& I, int n0, int rep, T bp, T bA, const C2<T>* __restrict__ psi,
                                              const T* __restrict__ ab, const T* __restrict__ abei,
                                              const C2<T>* __restrict__ U, const C2<T>* __restrict__ G,
                                              const T* __restrict__ GA, const C2<T>* __restrict__ dO,
                                              const T* __restrict__ dAO, C2<T>* __restrict__ dN,
                                              T* __restrict__ dAN, T (&c)[17]) {
    const Geo g = I.g;
    const TableLinks<T> lk{U};
    auto dpsi = [&](int m) -> C2<T> {
        const C2<T> o = dO[m], gg = G[m];
        return cmk<T>(bp * o.x - gg.x, bp * o.y - gg.y);
    };
    auto dA = [&](int m) -> T { return bA * dAO[m] - GA[m]; };
    auto psi_at = [&](int m) -> C2<T> { return psi[m]; };
    auto phase = [&](int l) -> T { return link_phase(abei, ab, l); };
    const T eps0 = gsel<T>(I.epsilon, I.fepsilon), H = gsel<T>(I.H, I.fH);
#pragma unroll kCoefUnroll
    for (int r = 0; r < rep; ++r) {
        const int n = n0 + threadIdx.x + r * kThreads;
        cg_prefetch_ahead(r, rep, [&](int q) { coef_prefetch<T>(I, g, n0 + threadIdx.x + q * kThreads, psi, U, G, dO, ab, GA, dAO); });
        if (n < g.N) {
            const int i = n % g.Nx, j = n / g.Nx;
            const unsigned cb = I.cbits[n];
            if (SA) {
                coef_node<T, 17>(g, gsel<T>(I.kappa2, I.fkappa2), eps0, (const T*)I.eps_sp, H, psi_at, phase, ab, lk,
                                 n, i, j, cb, dpsi, dA, c);
            } else {
                T c5[5] = {T(0), T(0), T(0), T(0), T(0)};
                coef_node<T, 5>(g, T(-1), eps0, (const T*)I.eps_sp, H, psi_at, phase, ab, lk, n, i, j, cb, dpsi, dA,
                                c5);
                c[0] += c5[0]; c[5] += c5[1]; c[10] += c5[2]; c[15] += c5[3]; c[16] += c5[4];
            }
            dN[n] = dpsi(n);
            if (SA) {
                if (i < g.Nx - 1) { const int na = i + (g.Nx - 1) * j; dAN[na] = dA(na); }
                if (j < g.Ny - 1) { const int nb = g.Na + i + g.Nx * j; dAN[nb] = dA(nb); }
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? GLGPU_CG_MINB_COEF : 1)
kb_dir_coef(const Inst* __restrict__ insts, const CGTile* __restrict__ tiles, double* __restrict__ partials,
            CGLoop* loop) {
    const CGTile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    CGState* cs = I.cg;
    if (*(volatile const int*)&cs->done) return;
    const int gi = cs->gi, di = cs->di, pi = cs->pi;
    T c[17];
#pragma unroll
    for (int k = 0; k < 17; ++k) c[k] = T(0);
    auto run = [&](auto sa) {
        dir_coef_tile<T, decltype(sa)::value>(I, t.n0, t.rep, (T)cs->beta_psi, (T)cs->beta_A, (const C2<T>*)I.psi[pi],
                                              (const T*)I.ab[I.solveA ? pi : 0], (const T*)I.abei, (const C2<T>*)I.U,
                                              (const C2<T>*)I.gpsi[gi], (const T*)I.gA[gi], (const C2<T>*)I.dpsi[di],
                                              (const T*)I.dA[di], (C2<T>*)I.dpsi[1 - di], (T*)I.dA[1 - di], c);
    };
    if (I.solveA) run(std::true_type{});
    else run(std::false_type{});
    double cs17[17];
    block_sum<17>(c, cs17);
    if (threadIdx.x == 0) store_partials<T>(cs17, 17, partials + (size_t)blockIdx.x * kPart);
    if (last_cta_of_instance(cs, I.ntiles)) inst_alpha<sizeof(T) == 8>(I, cs, partials, loop);
}

// energy-ratio stop, target stop, energy-window stop and iteration cap of one
// instance, by the CTA that finished its last tile.  The energy window: every
// `window` iterations the energy is compared with the last mark; if it fell by no
// more than wtol |E| over the window the instance stops (status 5), else the mark
// moves.  It ends runs whose gradient cannot reach its tolerance because the
// arithmetic's rounding floor is above it (FP32 stencils) once the energy has
// stopped improving.  No counterpart in the reference (its CG stops on the
// per-iteration energy ratio, cg.py:315-318).
__device__ __noinline__ void inst_energy_stop(const Inst& I, CGState* cs, const double* partials, CGLoop* loop) {
    __shared__ double e1[1];
    cta_tile_sums<1>(partials, I.tile0, I.ntiles, I.g.dxdy, e1);
    if (threadIdx.x != 0) return;
    const double E = e1[0];
    cs->E_prev = cs->E;
    cs->E = E;
    const int it = cs->iter;
    cs->iter = it + 1;
    int stop = 0;
    if (it > 0 && fabs(E / cs->E_prev - 1.0) < loop->rtol) {
        stop = 2;
    } else if (I.cg_target == I.cg_target && E <= I.cg_target + I.cg_target_tol * fabs(I.cg_target)) {
        stop = 4;
    } else if (loop->window > 0 && cs->iter - cs->it_mark >= loop->window) {
        if (cs->E_mark - E <= loop->wtol * fabs(E)) {
            stop = 5;
        } else {
            cs->E_mark = E;
            cs->it_mark = cs->iter;
        }
    }
    if (!stop && cs->iter >= loop->n_iter) stop = 3;
    if (stop) {
        cs->done = 1;
        cs->status = stop;
        atomicSub(&loop->active, 1);
    }
}

// step and energy of the new state of one tile
template <typename T, bool SA>
__device__ __forceinline__ void step_tile(const Inst& I, int n0, int rep, T ap, T aA, const C2<T>* __restrict__ psi,
                                          C2<T>* __restrict__ psiN, const C2<T>* __restrict__ dpsi,
                                          const T* __restrict__ ab, T* __restrict__ abN, const T* __restrict__ dA,
                                          const T* __restrict__ abei, C2<T>* __restrict__ U, T (&v)[1]) {
    const Geo g = I.g;
    auto psi_new = [&](int m) -> C2<T> {
        const C2<T> d = dpsi[m];
        C2<T> p = psi[m];
        p.x = ap * d.x + p.x;
        p.y = ap * d.y + p.y;
        return p;
    };
    auto ab_new = [&](int l) -> T { return aA * dA[l] + ab[l]; };
    const TableLinks<T> lk{U};
    const T k2 = gsel<T>(I.kappa2, I.fkappa2), eps0 = gsel<T>(I.epsilon, I.fepsilon), H = gsel<T>(I.H, I.fH);
#pragma unroll
    for (int r = 0; r < kCGRepMax; ++r) {
        if (r >= rep) break;
        const int n = n0 + threadIdx.x + r * kThreads;
        cg_prefetch_ahead(r, rep, [&](int q) { step_prefetch<T>(I, g, n0 + threadIdx.x + q * kThreads, psi, dpsi, ab, dA); });
        if (n < g.N) {
            const int i = n % g.Nx, j = n / g.Nx;
            if (SA) {
                if (i < g.Nx - 1) {
                    const int na = i + (g.Nx - 1) * j;
                    const T a = ab_new(na);
                    abN[na] = a;
                    U[na] = link_U<T>(GT(g, dx) * (abei ? abei[na] + a : a));
                }
                if (j < g.Ny - 1) {
                    const int nb = g.Na + i + g.Nx * j;
                    const T a = ab_new(nb);
                    abN[nb] = a;
                    U[nb] = link_U<T>(GT(g, dy) * (abei ? abei[nb] + a : a));
                }
            }
            // the node's own links' factors were written above by this thread
            v[0] += energy_density_f<T>(g, k2, eps0, (const T*)I.eps_sp, H, (unsigned)I.cbits[n], psi_new, abei,
                                        SA, ab_new, lk, n, i, j);
            psiN[n] = psi_new(n);
        }
    }
}

// Step psi += alpha_psi dpsi, A += alpha_A dA into the other state buffer (with
// the new link factors of the links a node owns), the energy of the new state
// per tile, and the instance's stop test in its last CTA.  Neighbour values of
// the new state are formed from the old buffer by the same arithmetic that their
// owners store, so the energy equals that of the stored state bit for bit.  The
// last CTA of the launch counts the active instances and sets the WHILE
// condition.
#ifndef GLGPU_CG_MINB_STEP
#define GLGPU_CG_MINB_STEP 4
#endif
template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? GLGPU_CG_MINB_STEP : 1)
kb_step(const Inst* __restrict__ insts, const CGTile* __restrict__ tiles, double* __restrict__ partials, CGLoop* loop,
        cudaGraphConditionalHandle cond, int use_cond) {
    const CGTile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    CGState* cs = I.cg;
    if (!*(volatile const int*)&cs->done) {
        const int pi = cs->pi, di = cs->di;
        T v[1] = {T(0)};
        auto run = [&](auto sa) {
            step_tile<T, decltype(sa)::value>(I, t.n0, t.rep, (T)cs->alpha_psi, (T)cs->alpha_A, (const C2<T>*)I.psi[pi],
                                              (C2<T>*)I.psi[1 - pi], (const C2<T>*)I.dpsi[di],
                                              (const T*)I.ab[I.solveA ? pi : 0], I.solveA ? (T*)I.ab[1 - pi] : nullptr,
                                              (const T*)I.dA[di], (const T*)I.abei, (C2<T>*)I.U, v);
        };
        if (I.solveA) run(std::true_type{});
        else run(std::false_type{});
        double vs[1];
        block_sum<1>(v, vs);
        if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kPart] = vs[0];
        if (last_cta_of_instance(cs, I.ntiles)) {
            inst_energy_stop(I, cs, partials, loop);
            if (threadIdx.x == 0) cs->pi = 1 - pi;
        }
    }
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&loop->ticket, 1) == (int)(gridDim.x - 1);
        if (s_last) {
            __threadfence();
            loop->ticket = 0;
            const int iters = loop->iters + 1;
            loop->iters = iters;
            const int act = atomicAdd(&loop->active, 0);
            const unsigned go = (act > 0 && iters < loop->n_iter + 2) ? 1u : 0u;
            if (use_cond) cudaGraphSetConditional(cond, go);
            loop->pad_ = (int)go;
        }
    }
}

// energy of the start state per tile (buffer 0)
template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_energy(const Inst* __restrict__ insts, const CGTile* __restrict__ tiles, double* __restrict__ partials) {
    const CGTile t = tiles[blockIdx.x];
    const int rep = t.rep;
    const Inst& I = insts[t.inst];
    const Geo g = I.g;
    const TableLinks<T> lk{(const C2<T>*)I.U};
    T v[1] = {T(0)};
#pragma unroll
    for (int r = 0; r < kCGRepMax; ++r) {
        if (r >= rep) break;
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

// end of a CG call: the state is copied back to buffer 0 where it ended in buffer 1
template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_finish(const Inst* __restrict__ insts, const CGTile* __restrict__ tiles) {
    const CGTile t = tiles[blockIdx.x];
    const int rep = t.rep;
    const Inst& I = insts[t.inst];
    if (I.cg->pi == 0) return;
    const Geo g = I.g;
#pragma unroll
    for (int r = 0; r < kCGRepMax; ++r) {
        if (r >= rep) break;
        const int n = t.n0 + threadIdx.x + r * kThreads;
        if (n >= g.N) break;
        ((C2<T>*)I.psi[0])[n] = ((const C2<T>*)I.psi[1])[n];
        if (I.solveA) {
            const int i = n % g.Nx, j = n / g.Nx;
            const T* src = (const T*)I.ab[1];
            T* dst = (T*)I.ab[0];
            if (i < g.Nx - 1) dst[i + (g.Nx - 1) * j] = src[i + (g.Nx - 1) * j];
            if (j < g.Ny - 1) dst[g.Na + i + g.Nx * j] = src[g.Na + i + g.Nx * j];
        }
    }
}

// start of a CG call: zero direction and gradient, the per-node cell bits (so
// the iteration kernels read one byte instead of four mask cells), the
// link-factor table of the start state (TableLinks), then the energy of the
// start state
template <typename T>
__global__ void __launch_bounds__(kThreads)
kb_zero_dir(const Inst* __restrict__ insts, const CGTile* __restrict__ tiles) {
    const CGTile t = tiles[blockIdx.x];
    const int rep = t.rep;
    const Inst& I = insts[t.inst];
    const Geo g = I.g;
#pragma unroll
    for (int r = 0; r < kCGRepMax; ++r) {
        if (r >= rep) break;
        const int n = t.n0 + threadIdx.x + r * kThreads;
        if (n >= g.N) break;
        ((C2<T>*)I.dpsi[0])[n] = cmk<T>(T(0), T(0));
        ((C2<T>*)I.gpsi[0])[n] = cmk<T>(T(0), T(0));
        const int i = n % g.Nx, j = n / g.Nx;
        I.cbits[n] = (uint8_t)cell_bits(g, I.mt, i, j);
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
        double e1[1];
        warp_tile_sums<1>(partials, I.tile0, I.ntiles, e1);
        const double E = e1[0] * I.g.dxdy;
        if ((threadIdx.x & 31) != 0) continue;
        CGState* cs = I.cg;
        cs->beta_psi = cs->beta_A = 0.0;
        cs->alpha_psi = cs->alpha_A = 0.0;
        cs->E = E;
        cs->E_prev = E;
        cs->E_mark = E;
        cs->it_mark = 0;
        cs->g2 = cs->g2_0 = 0.0;
        cs->iter = 0;
        cs->done = 0;
        cs->gi = 0;
        cs->di = 0;
        cs->status = 0;
        cs->pi = 0;
        cs->ticket = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        loop->active = ninst;
        loop->iters = 0;
        loop->ticket = 0;
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
    const CGTile* tiles;
    double* partials;
    CGLoop* loop;
    int ninst, ntiles, dtype;
};

#define CG_FN(name) \
    static void* fn_##name(int dt) { return dt == 8 ? (void*)kb_##name<double> : (void*)kb_##name<float>; }
CG_FN(grad)
CG_FN(dir_coef)
CG_FN(step)
CG_FN(energy)
CG_FN(zero_dir)
CG_FN(finish)
#undef CG_FN

static cudaError_t launch(void* fn, int grid, int block, void** args, cudaStream_t s) {
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, 0, s);
}

// Host-driven loop body (the graph holds the same launches).
static cudaError_t cg_launch_body(const CGLaunch& L, cudaStream_t s) {
    cudaGraphConditionalHandle none = 0;
    int zero = 0;
    const Inst* insts = L.insts;
    const CGTile* tiles = L.tiles;
    double* partials = L.partials;
    CGLoop* loop = L.loop;
    void* a[] = {&insts, &tiles, &partials, &loop};
    void* b[] = {&insts, &tiles, &partials, &loop, &none, &zero};
    cudaError_t e = launch(fn_grad(L.dtype), L.ntiles, kThreads, a, s);
    if (e == cudaSuccess) e = launch(fn_dir_coef(L.dtype), L.ntiles, kThreads, a, s);
    if (e == cudaSuccess) e = launch(fn_step(L.dtype), L.ntiles, kThreads, b, s);
    return e;
}

static cudaError_t cg_launch_prologue(const CGLaunch& L, cudaStream_t s) {
    const cudaGraphConditionalHandle none = 0;
    const Inst* insts = L.insts;
    const CGTile* tiles = L.tiles;
    double* partials = L.partials;
    void* a[] = {&insts, &tiles};
    void* b[] = {&insts, &tiles, &partials};
    cudaError_t e = launch(fn_zero_dir(L.dtype), L.ntiles, kThreads, a, s);
    if (e == cudaSuccess) e = launch(fn_energy(L.dtype), L.ntiles, kThreads, b, s);
    if (e != cudaSuccess) return e;
    kb_init<<<1, 1024, 0, s>>>(L.insts, L.ninst, L.partials, L.loop, none, 0);
    return cudaGetLastError();
}

static cudaError_t cg_launch_epilogue(const CGLaunch& L, cudaStream_t s) {
    const Inst* insts = L.insts;
    const CGTile* tiles = L.tiles;
    void* a[] = {&insts, &tiles};
    return launch(fn_finish(L.dtype), L.ntiles, kThreads, a, s);
}

#define GCHK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { err = e_; goto fail; } } while (0)

// The whole CG run of all instances as one graph:
//   zero_dir -> energy -> init -> WHILE(active) { grad -> dir_coef -> step } -> finish
static cudaError_t build_cg_graph(const CGLaunch& L, cudaGraphExec_t* exec) {
    cudaError_t err = cudaSuccess;
    cudaGraph_t top = nullptr, body = nullptr;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t prev = nullptr, nd, wh;
    int one = 1;
    const dim3 gt(L.ntiles), bt(kThreads), g1(1), b1(1024);
    const Inst* insts = L.insts;
    const CGTile* tiles = L.tiles;
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
        void* a[] = {&insts, &tiles, &partials};
        GCHK(add_kernel(top, &nd, &prev, 1, fn_energy(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &ninst, &partials, &loop, &h, &one};
        GCHK(add_kernel(top, &nd, &prev, 1, (void*)kb_init, g1, b1, a));
        prev = nd;
    }
    GCHK(add_while(top, &wh, &prev, 1, h, &body));
    {
        void* a[] = {&insts, &tiles};
        GCHK(add_kernel(top, &nd, &wh, 1, fn_finish(L.dtype), gt, bt, a));
    }
    prev = nullptr;
    {
        void* a[] = {&insts, &tiles, &partials, &loop};
        GCHK(add_kernel(body, &nd, nullptr, 0, fn_grad(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &tiles, &partials, &loop};
        GCHK(add_kernel(body, &nd, &prev, 1, fn_dir_coef(L.dtype), gt, bt, a));
        prev = nd;
    }
    {
        void* a[] = {&insts, &tiles, &partials, &loop, &h, &one};
        GCHK(add_kernel(body, &nd, &prev, 1, fn_step(L.dtype), gt, bt, a));
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

int batch_set_cg_window(glgpu_batch* b, int window, double rel_tol) {
    if (window < 0 || !(rel_tol >= 0.0)) return batch_error(b, GLGPU_E_ARG, "batch_set_cg_window: window < 0 or rel_tol < 0");
    b->cg_window = window;
    b->cg_window_tol = rel_tol;
    return GLGPU_OK;
}

int batch_cg(glgpu_batch* b, int n_iter, double rtol, double gtol, int flags, int32_t* iters, double* energies, double* grad_rel,
             int32_t* status, double* elapsed_ms) {
    if (n_iter < 0 || !(rtol >= 0.0) || !(gtol >= 0.0)) return batch_error(b, GLGPU_E_ARG, "batch_cg: bad n_iter, rtol or gtol");
    std::vector<Inst> insts(b->ninst);
    std::vector<CGTile> cgtiles;
    for (int q = 0; q < b->ninst; ++q) {
        glgpu_handle* h = b->hs[q];
        const int rc = cg_ensure(h);
        if (rc) return batch_error(b, rc, "batch_cg: " + h->last_error);
        cudaStreamSynchronize(h->stream);
        insts[q] = h->inst_h;
        // this copy of the descriptors indexes the CG tile table (rep x 256 nodes per tile)
        insts[q].tile0 = (int)cgtiles.size();
        const int rep = cg_rep_of(h->g.N);
        for (int n0 = 0; n0 < h->g.N; n0 += kThreads * rep) cgtiles.push_back(CGTile{q, n0, rep, 0});
        insts[q].ntiles = (int)cgtiles.size() - insts[q].tile0;
        insts[q].cg_exact = (flags & GLGPU_CG_EXACT_BOUNDARY) ? 1 : 0;
        insts[q].cg_target = b->cg_targets.empty() ? NAN : b->cg_targets[q];
        insts[q].cg_target_tol = b->cg_target_tol;
    }
    if (!b->cg_tiles) {
        b->cg_ntiles = (int)cgtiles.size();
        if (cudaMalloc(&b->cg_tiles, sizeof(CGTile) * cgtiles.size()) != cudaSuccess ||
            cudaMemcpy(b->cg_tiles, cgtiles.data(), sizeof(CGTile) * cgtiles.size(), cudaMemcpyHostToDevice) != cudaSuccess)
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
    lp.window = b->cg_window;
    lp.wtol = b->cg_window_tol;
    cudaError_t e = cudaMemcpyAsync(b->insts, insts.data(), sizeof(Inst) * insts.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->cg_loop, &lp, sizeof(lp), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return batch_error(b, GLGPU_E_CUDA, std::string("batch_cg: ") + cudaGetErrorString(e));
    CGLaunch L;
    L.insts = b->insts;
    L.tiles = (const CGTile*)b->cg_tiles;
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
        if (e == cudaSuccess) e = cg_launch_epilogue(L, s);
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
