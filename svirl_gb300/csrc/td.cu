// TDGL time stepping on the GPU: the Jacobi sweeps of the backward-Euler psi step
// and of the A step, and the time/Jacobi loops themselves, which run entirely on
// the device (a CUDA graph with nested conditional WHILE nodes; the sweep kernel
// that finishes last decides whether the loop continues).
//
// Reference: svirl/cuda/td.h:4-133 (psi sweep), td.h:310-463 (A sweep),
// svirl/solvers/td.py:157-218,252-325,342-377 (host loops, stop rule, swaps).
//
// Buffer rotation.  The reference copies psi into a separate right-hand-side
// buffer each step and ping-pongs psi/psi_next.  Here psi^(0) (the right-hand
// side) stays in buffer R and the other kFuse+1 buffers rotate: a launch reads
// psi^(k) and writes psi^(k+1) .. psi^(k+kFuse) (pbuf below), so no copy is
// needed, the loop can end after any sweep, and the values are those of the
// reference.  A uses three buffers, psi^(k) in (R+1+((k-1)&1))%3; this
// rotation also reproduces the reference's aliasing of the supercurrent
// argument (svirl/solvers/td.py:266,303): sweep k sees A^(2*floor(k/2)), which is
// buffer R for k<2 and (R+2)%3 afterwards; in odd sweeps that buffer is also the
// destination, read and then written by the same thread, as in the reference.
// The Langevin noise of sweep 0 (td.h:147-151,451-454) is recomputed in every
// sweep from its hash instead of being stored into the right-hand side.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "glgpu_bulk.cuh"
#include "glgpu_internal.h"

namespace glgpu {

__device__ __forceinline__ int buf_of(int R, int k) { return k == 0 ? R : (R + 1 + ((k - 1) & 1)) % 3; }

// Called by the last CTA of a launch: decide whether the Jacobi while loop goes on.
__device__ void finish_launch(LoopState* loop, cudaGraphConditionalHandle cond, int use_cond) {
    __threadfence();
    loop->blocks_done = 0u;
    int L = loop->launches + 1;
    loop->launches = L;
    loop->total_launches += 1;
    int act = atomicAdd(&loop->active, 0);
    int cont = act > 0 ? 1 : 0;
    if (cont && L >= loop->guard) {
        cont = 0;
        loop->err |= kErrLoopGuard;
    }
    loop->cont = cont;
    if (use_cond) cudaGraphSetConditional(cond, (unsigned)cont);
}

// Called by the CTA that finishes the last tile of an instance in an A sweep.
template <typename T>
__device__ void finish_instance_A(const Inst& I, LoopState* loop, int k) {
    InstState* st = I.st;
    __threadfence();
    unsigned long long b = atomicExch(&st->res, 0ull);
    T r = res_from_bits<T>(b);
    bool conv = jacobi_converged(r, I.stop_A);
    int s = k + 1;
    st->sweep = s;
    st->blocks_done = 0u;
    if (conv || s >= kMaxSweeps) {
        st->done = 1;
        // FP32: the buffers hold offsets from A^(0) (k_A_sweep); k_A_commit adds A^(0)
        if (sizeof(T) == 4) st->commitA = 1 + st->rhsA;
        st->rhsA = buf_of(st->rhsA, s);
        st->last_sweeps_A = s;
        st->total_sweeps_A += s;
        if (s > st->max_sweeps_A) st->max_sweeps_A = s;
        atomicSub(&loop->active, 1);
    }
}

// Buffer of psi^(s) in a psi Jacobi loop whose right-hand side psi^(0) is in
// buffer R: the kFuse + 1 other buffers rotate, so the input of a launch and its
// kFuse outputs are always distinct.
__device__ __forceinline__ int pbuf(int R, int s) { return s == 0 ? R : (R + 1 + (s - 1) % (kFuse + 1)) % kPsiBufs; }

// Called by the warp that finishes the last strip of an instance in a psi
// launch that did sweeps k+1 .. k+kFuse: the loop stops after the first of them
// that meets the reference's stop rule (or reaches the sweep cap), exactly where
// a loop of single sweeps stops; that sweep's output buffer becomes the state.
template <typename T>
__device__ void finish_instance_psi(const Inst& I, LoopState* loop, int k) {
    InstState* st = I.st;
    __threadfence();
    T r[kFuse];
#pragma unroll
    for (int l = 0; l < kFuse; ++l) r[l] = res_from_bits<T>(atomicExch(&st->resp[l], 0ull));
    const int nl = atomicExch(&st->nanlv, 0);
    int stop = 0;
#pragma unroll
    for (int l = kFuse; l >= 1; --l)
        if (jacobi_converged(r[l - 1], I.stop_psi) || k + l >= kMaxSweeps) stop = l;
    const int upto = stop ? stop : kFuse;
    if (nl & ((1 << upto) - 1)) st->nan_seen = 1;
    st->blocks_done = 0u;
    if (stop) {
        const int s = k + stop;
        st->sweep = s;
        st->done = 1;
        st->rhs = pbuf(st->rhs, s);
        st->last_sweeps_psi = s;
        st->total_sweeps_psi += s;
        if (s > st->max_sweeps_psi) st->max_sweeps_psi = s;
        atomicSub(&loop->active, 1);
    } else {
        st->sweep = k + kFuse;
    }
}

template <typename T>
__device__ __forceinline__ T block_max_res(T v, bool nan) {
    __shared__ T sm[kWarps];
    __shared__ int snan;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) snan = 0;
    v = warp_max(v);
    __syncthreads();
    if (nan) snan = 1;
    if (lane == 0) sm[w] = v;
    __syncthreads();
    if (tid == 0) {
        for (int q = 1; q < kWarps; ++q) v = v > sm[q] ? v : sm[q];
        if (snan) v = -v - T(1);  // flag NaN in the sign: residuals are >= 0
    }
    return v;
}

// Residual bookkeeping of one warp for the instance it is working on: per fused
// sweep, the warp max goes to the instance with one atomic, and the warp that
// completes the instance's last strip closes the launch for that instance.
template <typename T>
__device__ __forceinline__ void warp_flush(const Inst* insts, int inst, int k, const T (&wmax)[kFuse],
                                           const bool (&wnan)[kFuse], int count, LoopState* loop) {
    const unsigned full = 0xffffffffu;
    T m[kFuse];
    int nanbits = 0;
#pragma unroll
    for (int l = 0; l < kFuse; ++l) {
        m[l] = warp_max(wmax[l]);
        if (__any_sync(full, wnan[l])) nanbits |= 1 << l;
    }
    if ((threadIdx.x & 31) == 0 && count > 0) {
        const Inst& I = insts[inst];
        InstState* st = I.st;
        if (nanbits) atomicOr(&st->nanlv, nanbits);
#pragma unroll
        for (int l = 0; l < kFuse; ++l) atomicMax(&st->resp[l], res_bits(m[l]));
        __threadfence();
        unsigned prev = atomicAdd(&st->blocks_done, (unsigned)count);
        if (prev + (unsigned)count == (unsigned)I.nitems) finish_instance_psi<T>(I, loop, k);
    }
}

template <typename T> __device__ __forceinline__ C2<T> shfl_up_c(C2<T> v, int d) {
    return cmk<T>(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
template <typename T> __device__ __forceinline__ C2<T> shfl_down_c(C2<T> v, int d) {
    return cmk<T>(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}

// The backward-Euler Jacobi update of one node (svirl/cuda/td.h:4-133 with the
// Winecki-Adams link weights of td.h:159-163, coded as bits of cd: 0 left,
// 1 right, 2 lower, 3 upper link), in two parts.  The diagonal depends only on
// the right-hand side (with the Langevin term, rq), the linear coefficient and
// the link weights, which are fixed during a Jacobi loop, so its reciprocal is
// formed once per node and launch (psi_diag_inv) and each sweep only forms the
// neighbour sums (psi_node).  A node with neither a left nor a right link gets 0.
// The link table holds U scaled by dt/dx^2 (x links) or dt/dy^2 (y links), and
// 0 on links of weight 0, so the neighbour sum is one FMA chain per component
// with no branch per link.
template <typename T>
__device__ __forceinline__ T psi_diag_inv(C2<T> rq, T eps, unsigned cd, T dt, T idx2, T idy2) {
    // FP64: the link-count terms by selects, keeping conversions off the FP64 pipe
    if constexpr (sizeof(T) == 8) {
        const unsigned nx = (cd & 1u) + ((cd >> 1) & 1u), ny = ((cd >> 2) & 1u) + ((cd >> 3) & 1u);
        const T cx = nx == 0u ? T(0) : (nx == 1u ? idx2 : idx2 + idx2);
        const T cy = ny == 0u ? T(0) : (ny == 1u ? idy2 : idy2 + idy2);
        const T diag = T(1) + dt * (rq.x * rq.x + rq.y * rq.y - eps + (cx + cy));
        return T(1) / diag;
    } else {
        const bool rm0 = cd & 1u, rp0 = cd & 2u, r0m = cd & 4u, r0p = cd & 8u;
        const T wx = T(rm0) + T(rp0), wy = T(r0m) + T(r0p);
        const T diag = T(1) + dt * (rq.x * rq.x + rq.y * rq.y - eps + (idx2 * wx + idy2 * wy));
        return T(1) / diag;
    }
}

// rq + conj(ua_left) p_left + ua p_right + conj(ub_down) p_prev + ub p_next as one
// FMA chain per component, the link factors already scaled; p_next, the row the
// previous sweep produced last, enters at the end of the chain.
template <typename T>
__device__ __forceinline__ C2<T> psi_node(C2<T> p_left, C2<T> p_right, C2<T> p_prev, C2<T> p_next, C2<T> ua_left,
                                          C2<T> ua, C2<T> ub_down, C2<T> ub, C2<T> rq, T inv, unsigned cd) {
    const C2<T> z = cmk<T>(T(0), T(0));
    C2<T> out = z;
    T ax = fma(ua_left.x, p_left.x, rq.x);
    ax = fma(ua_left.y, p_left.y, ax);
    ax = fma(ua.x, p_right.x, ax);
    ax = fma(-ua.y, p_right.y, ax);
    T ay = fma(ua_left.x, p_left.y, rq.y);
    ay = fma(-ua_left.y, p_left.x, ay);
    ay = fma(ua.x, p_right.y, ay);
    ay = fma(ua.y, p_right.x, ay);
    ax = fma(ub_down.x, p_prev.x, ax);
    ax = fma(ub_down.y, p_prev.y, ax);
    ax = fma(ub.x, p_next.x, ax);
    ax = fma(-ub.y, p_next.y, ax);
    ay = fma(ub_down.x, p_prev.y, ay);
    ay = fma(-ub_down.y, p_prev.x, ay);
    ay = fma(ub.x, p_next.y, ay);
    ay = fma(ub.y, p_next.x, ay);
    const T vx = ax * inv, vy = ay * inv;
    if (cd & 3u) out = cmk<T>(vx, vy);
    return out;
}

// Per-row inputs of the psi update besides psi itself, as loaded: the link
// factors of the x link and the y link that start at the node, the right-hand
// side, the linear coefficient and the link-weight code ...
template <typename T> struct PsiSide {
    C2<T> ua, ub, rr;
    T eps;
    unsigned cd;
};
// ... and as used by the sweeps: rq = right-hand side with the Langevin term,
// inv = reciprocal of the diagonal.
template <typename T> struct PsiRow {
    C2<T> ua, ub, rq;
    T inv;
    unsigned cd;
};

// kFuse Jacobi sweeps of the psi step (svirl/cuda/td.h:4-133) over every active
// instance in one launch, reading the per-step tables of k_link_U (link factors
// U and link-weight codes), so the sweep does no transcendental math and no mask
// logic.  A warp owns a strip of kStripCols output columns and RR rows;
// its 32 lanes hold the columns x0-kFuse .. x0+31-kFuse, and sweep l (1..kFuse)
// is valid on lanes l..31-l, so the halo columns are recomputed in registers
// instead of being exchanged.  The warp walks down the rows: at step s it loads
// row j0-kFuse+s of psi^(k) and the per-row inputs one row behind, and sweep l
// produces row j0-kFuse+s-l from the three newest rows of sweep l-1 (each level
// lags the previous one by a row).  x neighbours come from the adjacent lanes.
// Every sweep's values on the strip are stored, and its residual kept, so the
// loop can stop after any of the fused sweeps.  The row walk is unrolled with
// every load issued one step ahead of its use.  Persistent grid: warps stride
// over the item table.
// CTAs of the psi sweep are small: its warps are independent, and registers are
// allocated per CTA, so small CTAs fill an SM with more warps.
#ifndef GLGPU_PSI_THREADS
#define GLGPU_PSI_THREADS 64
#endif
// CTAs per SM the register allocation must allow: FP32 at 8 (128 registers a
// thread, 16 warps per SM), FP64 at 1 (its sweep needs about 190 registers)
#ifndef GLGPU_PSI_MIN_CTAS_F32
#define GLGPU_PSI_MIN_CTAS_F32 8
#endif
#ifndef GLGPU_PSI_MIN_CTAS_F64
#define GLGPU_PSI_MIN_CTAS_F64 1
#endif
// Row steps of the strip walk unrolled together (0: the whole walk).
#ifndef GLGPU_PSI_ROW_UNROLL
#define GLGPU_PSI_ROW_UNROLL 0
#endif

// Rows of inputs loaded ahead of their use in the register-strip sweep: FP32 2
// (measured on 2049^2: 75 us per launch against 88 with 1 row; 3 rows: 76-77 us),
// FP64 1 (register bound).
#ifndef GLGPU_PSI_PREFETCH_F32
#define GLGPU_PSI_PREFETCH_F32 2
#endif
template <typename T> constexpr int kPFof = sizeof(T) == 4 ? GLGPU_PSI_PREFETCH_F32 : 1;
constexpr int kPsiThreads = GLGPU_PSI_THREADS, kPsiWarps = kPsiThreads / 32;
template <typename T> constexpr bool kStoreInv = sizeof(T) == 8;
template <typename T, int RR>
__global__ void __launch_bounds__(kPsiThreads, sizeof(T) == 4 ? GLGPU_PSI_MIN_CTAS_F32 : GLGPU_PSI_MIN_CTAS_F64)
k_psi_sweep(const Inst* __restrict__ insts, const Item* __restrict__ items, int nitems, LoopState* loop,
            cudaGraphConditionalHandle cond, int use_cond) {
    constexpr int K = kFuse, S = RR + 2 * kFuse, kPF = kPFof<T>;
    constexpr int kRowUnroll = GLGPU_PSI_ROW_UNROLL > 0 ? GLGPU_PSI_ROW_UNROLL : S;
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kPsiWarps + (threadIdx.x >> 5), nw = gridDim.x * kPsiWarps;
    int cur_inst = -1, k = 0, count = 0, done = 1;
    T wmax[K];
    bool wnan[K];
#pragma unroll
    for (int l = 0; l < K; ++l) {
        wmax[l] = T(0);
        wnan[l] = false;
    }
    // per-instance values, refreshed when the warp moves to another instance
    const C2<T>* cur = nullptr;
    const C2<T>* rhs = nullptr;
    C2<T>* outb[K];
    const C2<T>* U = nullptr;
    const uint8_t* code = nullptr;
    T* dinv = nullptr;
    uint32_t rt = 0;
    for (int it = gw; it < nitems; it += nw) {
        const Item w = items[it];
        if (w.inst < 0) continue;  // group padding
        if (w.inst != cur_inst) {
            if (cur_inst >= 0 && !done) warp_flush<T>(insts, cur_inst, k, wmax, wnan, count, loop);
            cur_inst = w.inst;
            const InstState* st = insts[cur_inst].st;
            done = *(volatile const int*)&st->done;
            k = *(volatile const int*)&st->sweep;
            const int R = *(volatile const int*)&st->rhs;
            rt = *(volatile const uint32_t*)&st->rand_t;
            const Inst& I = insts[cur_inst];
            cur = (const C2<T>*)I.psi[pbuf(R, k)];
            rhs = (const C2<T>*)I.psi[R];
#pragma unroll
            for (int l = 0; l < K; ++l) {
                outb[l] = (C2<T>*)I.psi[pbuf(R, k + 1 + l)];
                wmax[l] = T(0);
                wnan[l] = false;
            }
            U = (const C2<T>*)I.U;
            code = I.code;
            dinv = (T*)I.dinv;
            count = 0;
        }
        if (done) continue;
        const Inst& I = insts[cur_inst];
        const Geo g = I.g;
        const T* eps_sp = (const T*)I.eps_sp;
        const T dt = gsel<T>(I.dt, I.fdt), eps0 = gsel<T>(I.epsilon, I.fepsilon);
        const T idx2 = GT(g, idx2), idy2 = GT(g, idy2);
        const bool lang = I.lang_psi_on != 0;
        const T lc = gsel<T>(I.lang_psi, I.flang_psi);
        const int Nx = g.Nx, Ny = g.Ny;
        const int i = w.x0 - K + lane;
        const bool in_x = i >= 0 && i < Nx;
        const bool calc_lane = in_x && lane >= 1 && lane <= 30;        // lanes any sweep computes
        const bool own_lane = in_x && lane >= K && lane <= 31 - K;     // the strip's own columns
        const int j0 = w.j0;
        // FP64: the first launch of a step stores the diagonal reciprocals of the
        // strip's own nodes, later launches of the step load them (the diagonal is
        // fixed during the Jacobi loop; the FP64 pipe binds this build)
        const bool load_inv = kStoreInv<T> && k > 0, store_inv = kStoreInv<T> && k == 0;
        const C2<T> z = cmk<T>(T(0), T(0));
        auto load_psi = [&](int y) -> C2<T> { return (in_x && y >= 0 && y < Ny) ? __ldg(&cur[i + Nx * y]) : z; };
        auto load_side = [&](int y) -> PsiSide<T> {
            PsiSide<T> q;
            const bool row = y >= 0 && y < Ny;
            const int n = i + Nx * y;
            const bool ld = in_x && row, ldc = calc_lane && row;
            if constexpr (sizeof(T) == 4) {
                const float4 v = ld ? __ldg((const float4*)U + n) : make_float4(0.f, 0.f, 0.f, 0.f);
                q.ua = cmk<T>(v.x, v.y);
                q.ub = cmk<T>(v.z, v.w);
            } else {
                q.ua = ld ? __ldg(&U[2 * n]) : z;
                q.ub = ld ? __ldg(&U[2 * n + 1]) : z;
            }
            q.cd = ldc ? (unsigned)__ldg(&code[n]) : 0u;
            q.rr = ldc ? __ldg(&rhs[n]) : z;
            if (load_inv) q.eps = ldc ? __ldg(&dinv[n]) : T(0);  // the stored reciprocal
            else q.eps = (ldc && eps_sp) ? __ldg(&eps_sp[n]) : eps0;
            return q;
        };
        // window of sweep l-1 (l = 1..K) as seen by sweep l: rows y-1 and y
        C2<T> wp[K], wc[K];
        PsiRow<T> D[K + 1];  // D[m]: per-row inputs of row (j0 - K + s - 1) - m
#pragma unroll
        for (int l = 0; l < K; ++l) wp[l] = wc[l] = z;
#pragma unroll
        for (int m = 0; m <= K; ++m) D[m] = PsiRow<T>{z, z, z, T(0), 0u};
        // loaded inputs of row y -> sweep inputs (done one step after the loads were issued)
        auto finish_side = [&](const PsiSide<T>& q, int y) -> PsiRow<T> {
            PsiRow<T> r;
            r.ua = q.ua;
            r.ub = q.ub;
            r.cd = q.cd;
            r.rq = q.rr;
            if (lang && calc_lane && y >= 0 && y < Ny) {
                const uint32_t n = (uint32_t)(i + Nx * y);
                r.rq.x += lc * (rand_1<T>(n, rt) - T(0.5));
                r.rq.y += lc * (rand_2<T>(n, rt) - T(0.5));
            }
            if (load_inv) {
                r.inv = q.eps;
            } else {
                r.inv = (q.cd & 3u) ? psi_diag_inv<T>(r.rq, q.eps, q.cd, dt, idx2, idy2) : T(0);
                if (store_inv && own_lane && y >= j0 && y < j0 + RR && y < Ny) dinv[i + Nx * y] = r.inv;
            }
            return r;
        };
        // the rows' loads are issued kPF row steps ahead of their use (a ring of
        // kPF rows in registers; the walk is unrolled, so the indexing is static)
        C2<T> nx_p[kPF];
        PsiSide<T> nx_s[kPF];
#pragma unroll
        for (int a = 0; a < kPF; ++a) {
            nx_p[a] = load_psi(j0 - K + a);
            nx_s[a] = load_side(j0 - K - 1 + a);
        }
#pragma unroll kRowUnroll
        for (int s = 0; s < S; ++s) {
            C2<T> newrow = nx_p[s % kPF];  // psi^(k) on row j0 - K + s
#pragma unroll
            for (int m = K; m >= 1; --m) D[m] = D[m - 1];
            D[0] = finish_side(nx_s[s % kPF], j0 - K + s - 1);
            if (s + kPF < S) {
                nx_p[s % kPF] = load_psi(j0 - K + s + kPF);
                nx_s[s % kPF] = load_side(j0 - K - 1 + s + kPF);
            }
#pragma unroll
            for (int l = 1; l <= K; ++l) {
                C2<T> out = z;
                if (s >= 2 * l) {  // earlier rows of sweep l are above the strip's halo
                    const int y = j0 - K + s - l;
                    const C2<T> pc = wc[l - 1];
                    const C2<T> pl = shfl_up_c<T>(pc, 1), pr = shfl_down_c<T>(pc, 1);
                    const PsiRow<T>& d = D[l - 1];
                    const C2<T> ual = shfl_up_c<T>(d.ua, 1);
                    // every lane computes: outside the domain and on the edge lanes the
                    // loaded inputs are zero with code 0, and psi_node returns 0 there
                    {
                        out = psi_node<T>(pl, pr, wp[l - 1], newrow, ual, d.ua, D[l].ub, d.ub, d.rq, d.inv, d.cd);
                        if (own_lane && y >= j0 && y < j0 + RR && y < Ny) {
                            outb[l - 1][i + Nx * y] = out;
                            // max(|d re|, |d im|); a NaN component counts as 0 (the reference's
                            // int conversion).  FP64 compares the bit patterns (non-negative
                            // doubles order as integers), off the FP64 pipe; FP32 uses fmax,
                            // which drops NaN operands.
                            if constexpr (sizeof(T) == 8) {
                                const unsigned long long kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
                                unsigned long long bx = (unsigned long long)__double_as_longlong(out.x - pc.x) & kAbs;
                                unsigned long long by = (unsigned long long)__double_as_longlong(out.y - pc.y) & kAbs;
                                if ((bx > kInf) | (by > kInf)) wnan[l - 1] = true;
                                bx = bx > kInf ? 0ull : bx;
                                by = by > kInf ? 0ull : by;
                                const unsigned long long m = bx > by ? bx : by;
                                const unsigned long long w = (unsigned long long)__double_as_longlong(wmax[l - 1]);
                                wmax[l - 1] = __longlong_as_double((long long)(w > m ? w : m));
                            } else {
                                const T dr = fabs(out.x - pc.x), di = fabs(out.y - pc.y);
                                if (isnan(dr) | isnan(di)) wnan[l - 1] = true;
                                wmax[l - 1] = fmax(wmax[l - 1], fmax(dr, di));
                            }
                        }
                    }
                }
                // sweep l has used the window of sweep l-1: advance it by one row
                wp[l - 1] = wc[l - 1];
                wc[l - 1] = newrow;
                newrow = out;
            }
        }
        ++count;
    }
    if (cur_inst >= 0 && !done) warp_flush<T>(insts, cur_inst, k, wmax, wnan, count, loop);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned gdone = atomicAdd(&loop->blocks_done, 1u);
        if (gdone == gridDim.x - 1u) finish_launch(loop, cond, use_cond);
    }
}

// FP32 psi sweep with the inputs staged by bulk copies (TMA).  The same three
// fused Jacobi sweeps per launch and the same register walk down a strip as
// k_psi_sweep, bitwise the same values, but the rows a warp reads come from a
// ring of shared-memory stages filled by the copy engine several rows ahead,
// so the warps do not wait on global-memory latency.  A CTA runs kPsiGroup
// adjacent strips of one row band (one group of the item table); one thread
// (thread 0) copies, per row of the band, the group's columns x0 - 3 ..
// x0_last + 28 of psi^(k), of the right-hand side, of the link table and of the
// link-weight codes into the next free stage, each as one cp.async.bulk from the
// 16-byte boundary at or below the row segment (the arrays' row pitch, 8 Nx
// bytes, is not a multiple of 16 for odd Nx, so tensor maps cannot describe
// them).  Per stage a "full" mbarrier (the copies' bytes) and an "empty" one
// (one arrival per warp when the warp has read the stage).  Every wait is
// bounded; a wait that runs out sets kErrCopyWait in the loop state (the host
// reports it) and the CTA stops waiting.
constexpr int kBulkStages = 8, kBulkAhead = 5;  // ring depth, rows copied ahead of the one being used
static_assert(kBulkStages >= kBulkAhead + 3, "a stage is reused only after every warp released it");
constexpr int kBulkCols = kPsiGroup * kStripCols + 2 * kFuse;      // columns of a group's row
constexpr int kBulkPsiBytes = ((kBulkCols + 1) * 8 + 15) / 16 * 16;  // psi or rhs: one extra node of alignment
constexpr int kBulkUBytes = kBulkCols * 16;                         // (x link, y link) per node
constexpr int kBulkCodeBytes = (kBulkCols + 30) / 16 * 16;          // up to 15 bytes of alignment
constexpr int kBulkOffRhs = kBulkPsiBytes, kBulkOffU = 2 * kBulkPsiBytes, kBulkOffCode = kBulkOffU + kBulkUBytes;
constexpr int kBulkStageBytes = kBulkOffCode + kBulkCodeBytes;
constexpr int kBulkThreads = kPsiGroup * 32;
constexpr int kBulkSpins = 1 << 20;
static_assert(kBulkStageBytes % 16 == 0 && kBulkOffU % 16 == 0 && kBulkOffCode % 16 == 0, "stage layout");

#ifndef GLGPU_BULK_MIN_CTAS
#define GLGPU_BULK_MIN_CTAS 4
#endif
template <int RR>
__global__ void __launch_bounds__(kBulkThreads, GLGPU_BULK_MIN_CTAS)
k_psi_sweep_bulk(const Inst* __restrict__ insts, const Item* __restrict__ items, int nitems, LoopState* loop,
                 cudaGraphConditionalHandle cond, int use_cond) {
    using T = float;
    constexpr int K = kFuse, S = RR + 2 * kFuse, L = S + 1;  // row steps / rows copied per item
    __shared__ __align__(128) unsigned char ring[kBulkStages * kBulkStageBytes];
    __shared__ __align__(8) uint64_t full[kBulkStages], empty[kBulkStages];
    __shared__ int broken;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool leader = threadIdx.x == 0;
    if (leader) {
        for (int q = 0; q < kBulkStages; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], kPsiGroup);
        }
        broken = 0;
        fence_mbar_init();
    }
    __syncthreads();
    auto wait_bar = [&](uint64_t* bar, unsigned parity) {
        if (*(volatile int*)&broken) return;
        if (!mbar_wait(bar, parity, kBulkSpins)) {
            atomicOr(&loop->err, kErrCopyWait);
            *(volatile int*)&broken = 1;
        }
    };
    const int ngroups = nitems / kPsiGroup;
    uint32_t qb = 0;      // row copies of this CTA so far (the same count in every thread)
    uint32_t issued = 0;  // row copies issued (thread 0)
    int cur_inst = -1, k = 0, count = 0;
    T wmax[K];
    bool wnan[K];
#pragma unroll
    for (int l = 0; l < K; ++l) {
        wmax[l] = T(0);
        wnan[l] = false;
    }
    C2<T>* outb[K];
    uint32_t rt = 0;
    for (int gi = blockIdx.x; gi < ngroups; gi += gridDim.x) {
        const Item w0 = items[gi * kPsiGroup];
        const Item w = items[gi * kPsiGroup + wid];
        int last = 0;
#pragma unroll
        for (int t = 1; t < kPsiGroup; ++t)
            if (items[gi * kPsiGroup + t].inst >= 0) last = t;
        const int xl = items[gi * kPsiGroup + last].x0;
        const Inst& I = insts[w0.inst];
        const InstState* st = I.st;
        if (*(volatile const int*)&st->done) continue;  // this instance's loop has stopped
        const int kg = *(volatile const int*)&st->sweep;
        const int R = *(volatile const int*)&st->rhs;
        const Geo g = I.g;
        const int Nx = g.Nx, Ny = g.Ny;
        const C2<T>* cur = (const C2<T>*)I.psi[pbuf(R, kg)];
        const C2<T>* rhs = (const C2<T>*)I.psi[R];
        const float4* U = (const float4*)I.U;
        const uint8_t* code = I.code;
        const int ca = max(w0.x0 - K, 0), cb = min(xl + kStripCols + K - 1, Nx - 1);  // the group's columns
        const int j0 = w0.j0;
        // copy row r (0..L-1) of this item, row y = j0 - K - 1 + r, into the stage of copy number q
        auto issue = [&](uint32_t q, int r) {
            const int sidx = (int)(q % kBulkStages);
            if (q >= (uint32_t)kBulkStages) wait_bar(&empty[sidx], ((q / kBulkStages) + 1u) & 1u);
            const int y = j0 - K - 1 + r;
            unsigned char* stg = ring + sidx * kBulkStageBytes;
            if (y < 0 || y >= Ny) {
                mbar_arrive(&full[sidx]);  // nothing to copy: the readers use zeros outside the domain
                return;
            }
            const long long e0 = (long long)ca + (long long)Nx * y, e1 = (long long)cb + (long long)Nx * y;
            const long long p0 = e0 & ~1LL, p1 = (e1 + 2) & ~1LL;   // psi, rhs: 16-byte units
            const long long c0 = e0 & ~15LL, c1 = (e1 + 16) & ~15LL;  // codes: 16-byte units
            const unsigned pb = (unsigned)(p1 - p0) * 8u, ub = (unsigned)(e1 - e0 + 1) * 16u, cbts = (unsigned)(c1 - c0);
            mbar_arrive_expect_tx(&full[sidx], 2u * pb + ub + cbts);
            bulk_g2s(stg, cur + p0, pb, &full[sidx]);
            bulk_g2s(stg + kBulkOffRhs, rhs + p0, pb, &full[sidx]);
            bulk_g2s(stg + kBulkOffU, U + e0, ub, &full[sidx]);
            bulk_g2s(stg + kBulkOffCode, code + c0, cbts, &full[sidx]);
        };
        if (leader)
            for (int r = 0; r <= kBulkAhead && r < L; ++r) issue(issued++, r);
        const bool real = w.inst >= 0;
        if (real && w.inst != cur_inst) {
            if (cur_inst >= 0) warp_flush<T>(insts, cur_inst, k, wmax, wnan, count, loop);
            cur_inst = w.inst;
            k = kg;
            rt = *(volatile const uint32_t*)&st->rand_t;
#pragma unroll
            for (int l = 0; l < K; ++l) {
                outb[l] = (C2<T>*)I.psi[pbuf(R, k + 1 + l)];
                wmax[l] = T(0);
                wnan[l] = false;
            }
            count = 0;
        }
        const T* eps_sp = (const T*)I.eps_sp;
        const T dt = I.fdt, eps0 = I.fepsilon;
        const T idx2 = GT(g, idx2), idy2 = GT(g, idy2);
        const bool lang = I.lang_psi_on != 0;
        const T lc = I.flang_psi;
        const int i = w.x0 - K + lane;
        const bool in_x = real && i >= 0 && i < Nx;
        const bool calc_lane = in_x && lane >= 1 && lane <= 30;
        const bool own_lane = in_x && lane >= K && lane <= 31 - K;
        const int jw = w.j0;
        const int rel = i - ca;
        const C2<T> z = cmk<T>(T(0), T(0));
        auto psi_at = [&](const unsigned char* stg, int y) -> C2<T> {
            return (in_x && y >= 0 && y < Ny) ? ((const float2*)stg)[rel + ((ca + Nx * y) & 1)] : z;
        };
        auto side_at = [&](const unsigned char* stg, int y) -> PsiSide<T> {
            PsiSide<T> q;
            const bool row = y >= 0 && y < Ny;
            const bool ld = in_x && row, ldc = calc_lane && row;
            if (ld) {
                const float4 v = ((const float4*)(stg + kBulkOffU))[rel];
                q.ua = cmk<T>(v.x, v.y);
                q.ub = cmk<T>(v.z, v.w);
            } else {
                q.ua = q.ub = z;
            }
            q.cd = ldc ? (unsigned)stg[kBulkOffCode + rel + ((ca + Nx * y) & 15)] : 0u;
            q.rr = ldc ? ((const float2*)(stg + kBulkOffRhs))[rel + ((ca + Nx * y) & 1)] : z;
            q.eps = (ldc && eps_sp) ? __ldg(&eps_sp[i + Nx * y]) : eps0;
            return q;
        };
        auto finish_side = [&](const PsiSide<T>& q, int y) -> PsiRow<T> {
            PsiRow<T> r;
            r.ua = q.ua;
            r.ub = q.ub;
            r.cd = q.cd;
            r.rq = q.rr;
            if (lang && calc_lane && y >= 0 && y < Ny) {
                const uint32_t n = (uint32_t)(i + Nx * y);
                r.rq.x += lc * (rand_1<T>(n, rt) - T(0.5));
                r.rq.y += lc * (rand_2<T>(n, rt) - T(0.5));
            }
            r.inv = (q.cd & 3u) ? psi_diag_inv<T>(r.rq, q.eps, q.cd, dt, idx2, idy2) : T(0);
            return r;
        };
        auto stage = [&](uint32_t q) -> const unsigned char* { return ring + (int)(q % kBulkStages) * kBulkStageBytes; };
        auto parity = [&](uint32_t q) -> unsigned { return (q / kBulkStages) & 1u; };
        auto release = [&](uint32_t q) {
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[q % kBulkStages]);
        };
        C2<T> wp[K], wc[K];
        PsiRow<T> D[K + 1];
#pragma unroll
        for (int l = 0; l < K; ++l) wp[l] = wc[l] = z;
#pragma unroll
        for (int m = 0; m <= K; ++m) D[m] = PsiRow<T>{z, z, z, T(0), 0u};
        wait_bar(&full[qb % kBulkStages], parity(qb));
        // rolled: the stage index is dynamic anyway, and an unrolled walk with the
        // copy issue inlined in every step overflowed the instruction cache
#pragma unroll 1
        for (int s = 0; s < S; ++s) {
            if (leader && s + kBulkAhead + 1 < L) issue(issued++, s + kBulkAhead + 1);
            wait_bar(&full[(qb + s + 1) % kBulkStages], parity(qb + s + 1));
            C2<T> newrow = psi_at(stage(qb + s + 1), jw - K + s);  // psi^(k) on row jw - K + s
            const PsiSide<T> sd = side_at(stage(qb + s), jw - K + s - 1);
            release(qb + s);
#pragma unroll
            for (int m = K; m >= 1; --m) D[m] = D[m - 1];
            D[0] = finish_side(sd, jw - K + s - 1);
#pragma unroll
            for (int l = 1; l <= K; ++l) {
                C2<T> out = z;
                if (s >= 2 * l) {
                    const int y = jw - K + s - l;
                    const C2<T> pc = wc[l - 1];
                    const C2<T> pl = shfl_up_c<T>(pc, 1), pr = shfl_down_c<T>(pc, 1);
                    const PsiRow<T>& d = D[l - 1];
                    const C2<T> ual = shfl_up_c<T>(d.ua, 1);
                    out = psi_node<T>(pl, pr, wp[l - 1], newrow, ual, d.ua, D[l].ub, d.ub, d.rq, d.inv, d.cd);
                    if (own_lane && y >= jw && y < jw + RR && y < Ny) {
                        outb[l - 1][i + Nx * y] = out;
                        const T dr = fabs(out.x - pc.x), di = fabs(out.y - pc.y);
                        if (isnan(dr) | isnan(di)) wnan[l - 1] = true;
                        wmax[l - 1] = fmax(wmax[l - 1], fmax(dr, di));
                    }
                }
                wp[l - 1] = wc[l - 1];
                wc[l - 1] = newrow;
                newrow = out;
            }
        }
        release(qb + S);
        qb += L;
        if (real) ++count;
    }
    if (cur_inst >= 0) warp_flush<T>(insts, cur_inst, k, wmax, wnan, count, loop);
    // every copy issued was waited for; after a wait that ran out, give the
    // copies still in flight a bounded time to land before the CTA exits
    if (leader && *(volatile int*)&broken)
        for (uint32_t q = issued > (uint32_t)kBulkStages ? issued - kBulkStages : 0u; q < issued; ++q)
            mbar_wait(&full[q % kBulkStages], (q / kBulkStages) & 1u, kBulkSpins);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned gdone = atomicAdd(&loop->blocks_done, 1u);
        if (gdone == gridDim.x - 1u) finish_launch(loop, cond, use_cond);
    }
}

// Called by the CTA that finishes the last tile of an instance in a
// Crank-Nicolson psi sweep (one sweep per launch): the loop state keeps the max of
// the squared change, which the reference's Crank-Nicolson kernel puts into its
// residual code (svirl/cuda/td.h:285-291), so the usual stop predicate applies.
template <typename T>
__device__ void finish_instance_cn(const Inst& I, LoopState* loop, int k) {
    InstState* st = I.st;
    __threadfence();
    const T r2 = res_from_bits<T>(atomicExch(&st->res, 0ull));
    const bool conv = jacobi_converged(r2, I.stop_psi);
    const int s = k + 1;
    st->sweep = s;
    st->blocks_done = 0u;
    if (conv || s >= kMaxSweeps) {
        st->done = 1;
        st->rhs = pbuf(st->rhs, s);
        st->last_sweeps_psi = s;
        st->total_sweeps_psi += s;
        if (s > st->max_sweeps_psi) st->max_sweeps_psi = s;
        atomicSub(&loop->active, 1);
    }
}

// One Jacobi sweep of the Crank-Nicolson psi step of the reference's
// commented-out kernel (svirl/cuda/td.h:136-292; no host code of the reference
// launches it): half explicit, half implicit (c_lhs = c_rhs = 1/2), Du link
// weights r = (cell + cell) / 2 with ig = 4 / (r_m0 + r_p0 + r_0m + r_0p), the
// nonlinear coefficient |psi_rhs|^2 in both halves, and the squared change as the
// residual.  The explicit part of the links comes from the right-hand side on all
// four (the trapezoidal rule, `as_written` = 0) or, as the kernel writes it, on
// the left x link only and from psi^(k) on the other three (`as_written` = 1).  One thread per node;
// psi^(k) -> psi^(k+1) in the same rotating buffers as the backward-Euler sweep.
// The Langevin term of sweep 0 is recomputed from its hash for the node and its
// left neighbour in every sweep (the reference stores it into psi_rhs at sweep 0,
// where a thread may read its neighbour's value before or after that store).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_psi_sweep_cn(const Inst* __restrict__ insts, const Tile* __restrict__ tiles, LoopState* loop,
               cudaGraphConditionalHandle cond, int use_cond, int as_written) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    InstState* st = I.st;
    const int tid = threadIdx.x;
    __shared__ int s_skip, s_k, s_R, s_RA;
    __shared__ uint32_t s_rt;
    if (tid == 0) {
        s_skip = *(volatile int*)&st->done;
        s_k = *(volatile int*)&st->sweep;
        s_R = *(volatile int*)&st->rhs;
        s_RA = *(volatile int*)&st->rhsA;
        s_rt = *(volatile uint32_t*)&st->rand_t;
    }
    __syncthreads();
    if (!s_skip) {
        const int k = s_k, R = s_R;
        const C2<T>* __restrict__ cur = (const C2<T>*)I.psi[pbuf(R, k)];
        const C2<T>* __restrict__ rhs = (const C2<T>*)I.psi[R];
        C2<T>* nxt = (C2<T>*)I.psi[pbuf(R, k + 1)];
        const T* __restrict__ A = (const T*)I.ab[s_RA];
        const Geo g = I.g;
        const int n = t.n0 + tid;
        T res = T(0);
        bool nan = false;
        if (n < g.N) {
            const int i = n % g.Nx, j = n / g.Nx;
            const unsigned cb = cell_bits(g, I.mt, i, j);
            const bool mm = GL_MM(cb), mp = GL_MP(cb), pm = GL_PM(cb), pp = GL_PP(cb);
            const C2<T> p00 = cur[n];
            C2<T> v = cmk<T>(T(0), T(0));
            if (mm || mp || pm || pp) {
                const bool lang = I.lang_psi_on != 0;
                const T lc = gsel<T>(I.lang_psi, I.flang_psi);
                auto rq_at = [&](int m) -> C2<T> {
                    C2<T> r = rhs[m];
                    if (lang) {
                        r.x += lc * (rand_1<T>((uint32_t)m, s_rt) - T(0.5));
                        r.y += lc * (rand_2<T>((uint32_t)m, s_rt) - T(0.5));
                    }
                    return r;
                };
                const C2<T> rq = rq_at(n);
                const T dt = gsel<T>(I.dt, I.fdt);
                const T dx = GT(g, dx), dy = GT(g, dy), idx2 = GT(g, idx2), idy2 = GT(g, idy2);
                const T eps = I.eps_sp ? ((const T*)I.eps_sp)[n] : gsel<T>(I.epsilon, I.fepsilon);
                const T r_m0 = T(0.5) * (T(mm) + T(mp)), r_p0 = T(0.5) * (T(pm) + T(pp));
                const T r_0m = T(0.5) * (T(mm) + T(pm)), r_0p = T(0.5) * (T(mp) + T(pp));
                const T ig = T(4) / (r_m0 + r_p0 + r_0m + r_0p);
                const C2<T> z = cmk<T>(T(0), T(0));
                // r U psi^(k) on the links (implicit part) and r U psi_rhs (explicit part)
                C2<T> pm0 = z, pp0 = z, p0m = z, p0p = z, rm0 = z, rp0 = z, r0m = z, r0p = z;
                if (mm || mp) {
                    const C2<T> rU = cscale(r_m0, link_U<T>(-dx * A[(i - 1) + (g.Nx - 1) * j]));
                    pm0 = cmul(rU, cur[n - 1]);
                    rm0 = cmul(rU, rq_at(n - 1));
                }
                if (pm || pp) {
                    const C2<T> rU = cscale(r_p0, link_U<T>(dx * A[i + (g.Nx - 1) * j]));
                    pp0 = cmul(rU, cur[n + 1]);
                    rp0 = as_written ? pp0 : cmul(rU, rq_at(n + 1));
                }
                if (mm || pm) {
                    const C2<T> rU = cscale(r_0m, link_U<T>(-dy * A[g.Na + i + g.Nx * (j - 1)]));
                    p0m = cmul(rU, cur[n - g.Nx]);
                    r0m = as_written ? p0m : cmul(rU, rq_at(n - g.Nx));
                }
                if (mp || pp) {
                    const C2<T> rU = cscale(r_0p, link_U<T>(dy * A[g.Na + i + g.Nx * j]));
                    p0p = cmul(rU, cur[n + g.Nx]);
                    r0p = as_written ? p0p : cmul(rU, rq_at(n + g.Nx));
                }
                const T c = T(0.5);  // c_lhs = c_rhs
                const T a2 = rq.x * rq.x + rq.y * rq.y;
                const T lw = idx2 * (r_m0 + r_p0) + idy2 * (r_0m + r_0p);
                // explicit part: psi_rhs (1 - c dt (|psi_rhs|^2 - eps)) + c dt ig (idx2 (rhs_m0 + psi_p0)
                //   + idy2 (psi_0m + psi_0p) - lw psi_rhs); implicit part: c dt ig (idx2 (psi_m0 + psi_p0)
                //   + idy2 (psi_0m + psi_0p))
                const T e = T(1) - c * dt * (a2 - eps);
                const C2<T> ex = csub(cadd(cscale(idx2, cadd(rm0, rp0)), cscale(idy2, cadd(r0m, r0p))), cscale(lw, rq));
                const C2<T> im = cadd(cscale(idx2, cadd(pm0, pp0)), cscale(idy2, cadd(p0m, p0p)));
                const C2<T> num = cadd(cadd(cscale(e, rq), cscale(c * dt * ig, ex)), cscale(c * dt * ig, im));
                const T den = T(1) + c * dt * (a2 - eps + ig * lw);
                v = cmk<T>(num.x / den, num.y / den);
            }
            nxt[n] = v;
            const T dr = v.x - p00.x, di = v.y - p00.y;
            const T r2 = dr * dr + di * di;
            if (r2 == r2) res = r2; else nan = true;
        }
        T bmax = block_max_res<T>(res, nan);
        if (tid == 0) {
            if (bmax < T(0)) {
                atomicOr(&st->nan_seen, 1);
                bmax = -(bmax + T(1));
            }
            atomicMax(&st->res, res_bits(bmax));
            __threadfence();
            unsigned prev = atomicAdd(&st->blocks_done, 1u);
            if (prev == (unsigned)I.ntiles - 1u) finish_instance_cn<T>(I, loop, k);
        }
    }
    if (tid == 0) {
        __threadfence();
        unsigned gdone = atomicAdd(&loop->blocks_done, 1u);
        if (gdone == gridDim.x - 1u) finish_launch(loop, cond, use_cond);
    }
}

// One Jacobi sweep of the A step (svirl/cuda/td.h:310-463): each thread owns the
// x link and the y link that start at its node.  A CTA takes a 2-D tile of
// kATX x kATY nodes (ATile) and first stages the current iterate of the links its
// nodes read (x links of rows j0-1 .. j0+kATY and columns i0-1 .. i0+kATX-1, y links
// of rows j0-1 .. j0+kATY-1 and columns i0-1 .. i0+kATX) into shared memory with
// coalesced row loads; the twelve neighbour values of a node's two link updates
// then come from shared memory.  One prologue, one block reduction and one set of
// atomics per tile (2,048 nodes; per 256 they made each CTA's life a chain of
// dependent loads and atomics; that version took 0.202 ms per sweep at 2049^2,
// 0.125 ms with four 256-node tiles per CTA).  The arithmetic of a link is unchanged.
// resident CTAs per SM asked of the compiler for the FP32 A sweep (caps its registers)
#ifndef GLGPU_A_MINB
#define GLGPU_A_MINB 8
#endif
template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? GLGPU_A_MINB : 1)
k_A_sweep(const Inst* __restrict__ insts, const ATile* __restrict__ atiles, LoopState* loop,
          cudaGraphConditionalHandle cond, int use_cond) {
    const int tid = threadIdx.x;
    __shared__ int s_skip, s_k, s_R, s_P;
    __shared__ uint32_t s_rt;
    __shared__ T sx[kATY + 2][kATX + 1];
    __shared__ T sy[kATY + 1][kATX + 2];
    {
        const ATile t = atiles[blockIdx.x];
        const Inst& I = insts[t.inst];
        InstState* st = I.st;
        if (tid == 0) {
            s_skip = *(volatile int*)&st->done;
            s_k = *(volatile int*)&st->sweep;
            s_R = *(volatile int*)&st->rhsA;
            s_P = *(volatile int*)&st->rhs;
            s_rt = *(volatile uint32_t*)&st->rand_t;
        }
        __syncthreads();
        if (!s_skip) {
            const int k = s_k, R = s_R;
            // FP32: the iterates are offsets delta = A - A^(0) from the loop's right-hand
            // side (see the delta branch below); delta^(0) = 0
            constexpr bool kDelta = sizeof(T) == 4;
            const T* cur = (kDelta && k == 0) ? nullptr : (const T*)I.ab[buf_of(R, k)];
            const T* rhs = (const T*)I.ab[R];
            // with fixed vortices the supercurrent phases come from the irregular
            // potential buffer, which holds A_irr + A^(0) on its first N elements
            // (td.py:256-270), so there is no aliasing
            const T* abi = I.vpi ? (const T*)I.vpi : (const T*)I.ab[k < 2 ? R : (R + 2) % 3];
            T* nxt = (T*)I.ab[(R + 1 + (k & 1)) % 3];
            const C2<T>* __restrict__ psi = (const C2<T>*)I.psi[s_P];
            const Geo g = I.g;
            // the current iterate around the tile into shared memory (0 outside the domain;
            // those entries are never read)
            if (cur) {
                for (int e = tid; e < (kATY + 2) * (kATX + 1); e += kThreads) {
                    const int r = e / (kATX + 1), c = e - r * (kATX + 1);
                    const int i = t.i0 - 1 + c, j = t.j0 - 1 + r;
                    sx[r][c] = (i >= 0 && i < g.Nx - 1 && j >= 0 && j < g.Ny) ? cur[i + (g.Nx - 1) * j] : T(0);
                }
                for (int e = tid; e < (kATY + 1) * (kATX + 2); e += kThreads) {
                    const int r = e / (kATX + 2), c = e - r * (kATX + 2);
                    const int i = t.i0 - 1 + c, j = t.j0 - 1 + r;
                    sy[r][c] = (i >= 0 && i < g.Nx && j >= 0 && j < g.Ny - 1) ? cur[g.Na + i + g.Nx * j] : T(0);
                }
            }
            __syncthreads();
            // x link (i, j) and y link (i, j) of the current iterate
            auto cx = [&](int i, int j) -> T { return sx[j - t.j0 + 1][i - t.i0 + 1]; };
            auto cy = [&](int i, int j) -> T { return sy[j - t.j0 + 1][i - t.i0 + 1]; };
            // Per link, the update is (X + dt rho k2 dd nbs(A^(k))) / D, where the fixed part
            // X (right-hand side, noise, boundary field, supercurrent) depends on k only
            // through the supercurrent argument A^(2 floor(k/2)) (the fixed-vortex potential
            // with fixed vortices, constant over the loop).  Sweeps that start a pair
            // (`fresh`) compute X and store it; the other sweeps of the pair read it back,
            // so the sincos, the psi loads and the right-hand side's neighbour loads are paid
            // once per two sweeps.  X (and in FP32 the A^(0) part G of X, constant over the
            // loop) live in the link-factor buffer U, which the A loop does not read and
            // k_link_U rebuilds before the next psi loop.  Both are stored rounded (mul_rn
            // keeps G out of a fused multiply-add), so a pair's two sweeps use equal values.
            const bool fresh = k == 0 || (!I.vpi && (k & 1) == 0);
            T* Xc = (T*)I.U;
            T* Gc = Xc + g.Nab;
            T res = T(0);
            bool nan = false;
            // the node loop compiled twice, for the sweeps that compute the fixed parts and
            // for those that read them back, so that the second keeps only its own values
            // in registers
            auto sweep_nodes = [&](auto fresh_tag) {
                constexpr bool kFresh = decltype(fresh_tag)::value;
                for (int q = 0; q < kATY / (kThreads / kATX); ++q) {
                    const int ti = t.i0 + (tid % kATX), tj = t.j0 + tid / kATX + (kThreads / kATX) * q;
                    const bool in = ti < g.Nx && tj < g.Ny;
                    const int n = in ? ti + g.Nx * tj : g.N;
                    T va = T(0), vb = T(0), ca = T(0), cbv = T(0);
                    bool has_a = false, has_b = false;
                    int na = 0, nb = 0;
                    if constexpr (kDelta) {
                        // The same Jacobi iteration as the FP64 branch, written for delta: with
                        // A^(k) = A^(0) + delta^(k) the update of a link is
                        //   delta' = (noise + dt rho (js + rh) + dt rho k2 (dd nbs(A^(0)) - 2 d^-2 A^(0))
                        //            + dt rho k2 dd nbs(delta^(k))) / D,
                        // and the stop rule's |A^(k+1) - A^(k)| = |delta^(k+1) - delta^(k)|.  In FP32 the
                        // iterates of A itself differ by whole units in the last place once |A| > 8
                        // (the Landau gauge reaches H L), which the absolute stop rule of 1e-6
                        // (svirl/solvers/td.py:53-57) never accepts; delta is small, so the loop
                        // converges.  The supercurrent phase is that of A^(0) + delta^(2 floor(k/2)).
                        // The division by a link's constant diagonal is a multiplication by
                        // its reciprocal here; FP64 divides as the reference does.
                        if (n < g.N) {
                            const int i = ti, j = tj;
                            const int Nxa = g.Nx - 1, Na = g.Na;
                            has_a = i < g.Nx - 1;
                            has_b = j < g.Ny - 1;
                            na = i + Nxa * j;
                            nb = Na + i + g.Nx * j;
                            auto dlx = [&](int ii, int jj) -> T { return cur ? cx(ii, jj) : T(0); };
                            auto dly = [&](int ii, int jj) -> T { return cur ? cy(ii, jj) : T(0); };
                            const T idx2 = GT(g, idx2), idy2 = GT(g, idy2), idxy = GT(g, idxy);
                            const T k2 = I.fkappa2;
                            const T dt_rho_k2 = I.fdt * I.frho * k2;
                            T xa = T(0), xb = T(0);
                            if constexpr (kFresh) {
                                const T* al = (I.vpi || k < 2) ? nullptr : (const T*)I.ab[(R + 2) % 3];  // delta of the phase
                                const T ph_a = has_a ? (I.vpi ? abi[na] : rhs[na] + (al ? al[na] : T(0))) : T(0);
                                const T ph_b = has_b ? (I.vpi ? abi[nb] : rhs[nb] + (al ? al[nb] : T(0))) : T(0);
                                const unsigned cb = cell_bits(g, I.mt, i, j);
                                const C2<T> psi0 = psi[n];
                                const T dx = GT(g, dx), dy = GT(g, dy);
                                const T idx = GT(g, idx), idy = GT(g, idy);
                                const T H = I.fH;
                                const T dt_rho = I.fdt * I.frho;
                                const T lc = I.flang_A;
                                const bool lang = I.lang_A_on != 0;
                                if (has_a) {
                                    const T noise = lang ? lc * (rand_1<T>((uint32_t)na, s_rt) - T(0.5)) : T(0);
                                    T rh = T(0), dd = T(1);
                                    if (j == 0) { rh = T(2) * k2 * H * idy; dd = T(2); }
                                    else if (j == g.Ny - 1) { rh = -T(2) * k2 * H * idy; dd = T(2); }
                                    T jl = T(0);
                                    if (GL_PM(cb) || GL_PP(cb)) jl = idx * js_of<T>(psi0, dx * ph_a, psi[n + 1]);
                                    T ga;
                                    if (k == 0) {
                                        T nr = T(0);
                                        if (j > 0)
                                            nr += idy2 * rhs[i + Nxa * (j - 1)] - idxy * rhs[Na + i + g.Nx * (j - 1)] +
                                                  idxy * rhs[Na + i + 1 + g.Nx * (j - 1)];
                                        if (j < g.Ny - 1)
                                            nr += idy2 * rhs[i + Nxa * (j + 1)] + idxy * rhs[Na + i + g.Nx * j] - idxy * rhs[Na + i + 1 + g.Nx * j];
                                        ga = mul_rn<T>(dt_rho_k2, dd * nr - T(2) * idy2 * rhs[na]);
                                        Gc[na] = ga;
                                    } else {
                                        ga = Gc[na];
                                    }
                                    xa = noise + dt_rho * (jl + rh) + ga;
                                    Xc[na] = xa;
                                }
                                if (has_b) {
                                    const T noise = lang ? lc * (rand_2<T>((uint32_t)nb, s_rt) - T(0.5)) : T(0);
                                    T rh = T(0), dd = T(1);
                                    if (i == 0) { rh = -T(2) * k2 * H * idx; dd = T(2); }
                                    else if (i == g.Nx - 1) { rh = T(2) * k2 * H * idx; dd = T(2); }
                                    T jl = T(0);
                                    if (GL_MP(cb) || GL_PP(cb)) jl = idy * js_of<T>(psi0, dy * ph_b, psi[n + g.Nx]);
                                    T gb;
                                    if (k == 0) {
                                        T nr = T(0);
                                        if (i > 0)
                                            nr += idx2 * rhs[Na + (i - 1) + g.Nx * j] - idxy * rhs[(i - 1) + Nxa * j] + idxy * rhs[(i - 1) + Nxa * (j + 1)];
                                        if (i < g.Nx - 1)
                                            nr += idx2 * rhs[Na + (i + 1) + g.Nx * j] + idxy * rhs[i + Nxa * j] - idxy * rhs[i + Nxa * (j + 1)];
                                        gb = mul_rn<T>(dt_rho_k2, dd * nr - T(2) * idx2 * rhs[nb]);
                                        Gc[nb] = gb;
                                    } else {
                                        gb = Gc[nb];
                                    }
                                    xb = noise + dt_rho * (jl + rh) + gb;
                                    Xc[nb] = xb;
                                }
                            } else {
                                if (has_a) xa = Xc[na];
                                if (has_b) xb = Xc[nb];
                            }
                            if (has_a) {
                                const T dd = (j == 0 || j == g.Ny - 1) ? T(2) : T(1);
                                T nd = T(0);
                                if (j > 0) nd += idy2 * dlx(i, j - 1) - idxy * dly(i, j - 1) + idxy * dly(i + 1, j - 1);
                                if (j < g.Ny - 1) nd += idy2 * dlx(i, j + 1) + idxy * dly(i, j) - idxy * dly(i + 1, j);
                                va = (xa + dt_rho_k2 * dd * nd) * (T(1) / (T(1) + T(2) * dt_rho_k2 * idy2));
                                ca = dlx(i, j);
                            }
                            if (has_b) {
                                const T dd = (i == 0 || i == g.Nx - 1) ? T(2) : T(1);
                                T nd = T(0);
                                if (i > 0) nd += idx2 * dly(i - 1, j) - idxy * dlx(i - 1, j) + idxy * dlx(i - 1, j + 1);
                                if (i < g.Nx - 1) nd += idx2 * dly(i + 1, j) + idxy * dlx(i, j) - idxy * dlx(i, j + 1);
                                vb = (xb + dt_rho_k2 * dd * nd) * (T(1) / (T(1) + T(2) * dt_rho_k2 * idx2));
                                cbv = dly(i, j);
                            }
                        }
                    } else
                    if (n < g.N) {
                        const int i = ti, j = tj;
                        const int Nxa = g.Nx - 1, Na = g.Na;
                        has_a = i < g.Nx - 1;
                        has_b = j < g.Ny - 1;
                        na = i + Nxa * j;
                        nb = Na + i + g.Nx * j;
                        const T idx2 = GT(g, idx2), idy2 = GT(g, idy2), idxy = GT(g, idxy);
                        const T k2 = gsel<T>(I.kappa2, I.fkappa2);
                        const T dt_rho = gsel<T>(I.dt, I.fdt) * gsel<T>(I.rho, I.frho);
                        const T dt_rho_k2 = dt_rho * k2;
                        T xa = T(0), xb = T(0);
                        if constexpr (kFresh) {
                            // read the supercurrent phases before anything is stored (aliasing, see top)
                            const T ph_a = has_a ? abi[na] : T(0);
                            const T ph_b = has_b ? abi[nb] : T(0);
                            const unsigned cb = cell_bits(g, I.mt, i, j);
                            const C2<T> psi0 = psi[n];
                            const T dx = GT(g, dx), dy = GT(g, dy);
                            const T idx = GT(g, idx), idy = GT(g, idy);
                            const T H = gsel<T>(I.H, I.fH);
                            const T lc = gsel<T>(I.lang_A, I.flang_A);
                            const bool lang = I.lang_A_on != 0;
                            if (has_a) {
                                T r = rhs[na];
                                if (lang) r += lc * (rand_1<T>((uint32_t)na, s_rt) - T(0.5));
                                T rh = T(0);
                                if (j == 0) rh = T(2) * k2 * H * idy;
                                else if (j == g.Ny - 1) rh = -T(2) * k2 * H * idy;
                                T jl = T(0);
                                if (GL_PM(cb) || GL_PP(cb)) jl = idx * js_of<T>(psi0, dx * ph_a, psi[n + 1]);
                                xa = r + dt_rho * (jl + rh);
                                Xc[na] = xa;
                            }
                            if (has_b) {
                                T r = rhs[nb];
                                if (lang) r += lc * (rand_2<T>((uint32_t)nb, s_rt) - T(0.5));
                                T rh = T(0);
                                if (i == 0) rh = -T(2) * k2 * H * idx;
                                else if (i == g.Nx - 1) rh = T(2) * k2 * H * idx;
                                T jl = T(0);
                                if (GL_MP(cb) || GL_PP(cb)) jl = idy * js_of<T>(psi0, dy * ph_b, psi[n + g.Nx]);
                                xb = r + dt_rho * (jl + rh);
                                Xc[nb] = xb;
                            }
                        } else {
                            if (has_a) xa = Xc[na];
                            if (has_b) xb = Xc[nb];
                        }
                        if (has_a) {
                            const T dd = (j == 0 || j == g.Ny - 1) ? T(2) : T(1);
                            T nbs = T(0);
                            if (j > 0) nbs += idy2 * cx(i, j - 1) - idxy * cy(i, j - 1) + idxy * cy(i + 1, j - 1);
                            if (j < g.Ny - 1) nbs += idy2 * cx(i, j + 1) + idxy * cy(i, j) - idxy * cy(i + 1, j);
                            va = (xa + dt_rho_k2 * dd * nbs) / (T(1) + T(2) * dt_rho_k2 * idy2);
                            ca = cx(i, j);
                        }
                        if (has_b) {
                            const T dd = (i == 0 || i == g.Nx - 1) ? T(2) : T(1);
                            T nbs = T(0);
                            if (i > 0) nbs += idx2 * cy(i - 1, j) - idxy * cx(i - 1, j) + idxy * cx(i - 1, j + 1);
                            if (i < g.Nx - 1) nbs += idx2 * cy(i + 1, j) + idxy * cx(i, j) - idxy * cx(i, j + 1);
                            vb = (xb + dt_rho_k2 * dd * nbs) / (T(1) + T(2) * dt_rho_k2 * idx2);
                            cbv = cy(i, j);
                        }
                    }
                    if (n < g.N) {
                        if (has_a) {
                            nxt[na] = va;
                            T d = fabs(va - ca);
                            if (d == d) { if (d > res) res = d; } else nan = true;
                        }
                        if (has_b) {
                            nxt[nb] = vb;
                            T d = fabs(vb - cbv);
                            if (d == d) { if (d > res) res = d; } else nan = true;
                        }
                    }
                }
            };
            if (fresh) sweep_nodes(std::true_type{});
            else sweep_nodes(std::false_type{});
            T bmax = block_max_res<T>(res, nan);
            if (tid == 0) {
                if (bmax < T(0)) {
                    atomicOr(&st->nan_seen, 1);
                    bmax = -(bmax + T(1));
                }
                atomicMax(&st->res, res_bits(bmax));
                __threadfence();
                unsigned prev = atomicAdd(&st->blocks_done, 1u);
                if (prev + 1u == (unsigned)I.natiles) finish_instance_A<T>(I, loop, k);
            }
        }
    }
    if (tid == 0) {
        __threadfence();
        unsigned gdone = atomicAdd(&loop->blocks_done, 1u);
        if (gdone == gridDim.x - 1u) finish_launch(loop, cond, use_cond);
    }
}

// Tiles per CTA of the per-call kernels k_link_U and k_canonical_copy.  With one
// 256-node tile per CTA (16,401 CTAs at 2049^2) each CTA's life is a chain of
// dependent loads (tile, instance, state word, data) and the launch is bound by
// that latency; a CTA that takes kCallTiles consecutive tiles of one instance
// loads the instance and state once and issues the data loads of its kCallTiles
// nodes per thread together.  Tiles of several instances (a batch's boundaries)
// are taken one after the other.  Results do not depend on it.
constexpr int kCallTiles = 4;
static inline unsigned call_grid(int ntiles) { return (unsigned)((ntiles + kCallTiles - 1) / kCallTiles); }

// the tiles of CTA blockIdx.x (inst = -1 past the end); true when all of them
// that exist belong to one instance
__device__ __forceinline__ bool call_tiles(const Tile* __restrict__ tiles, int ntiles, Tile (&t)[kCallTiles]) {
#pragma unroll
    for (int q = 0; q < kCallTiles; ++q) {
        const int b = (int)blockIdx.x * kCallTiles + q;
        t[q] = b < ntiles ? tiles[b] : Tile{-1, 0};
    }
    bool same = true;
#pragma unroll
    for (int q = 1; q < kCallTiles; ++q) same = same && (t[q].inst < 0 || t[q].inst == t[0].inst);
    return same;
}

// Per-step tables of the psi Jacobi loop, during which A is fixed: the link
// factors U = exp(-i d a) of the current A times dt/d^2 (0 on links whose
// weight is 0), stored per node as the pair (x link, y link) that starts there,
// so a lane loads both with one 16-byte load (the CG fills the same buffer with
// its own unscaled factors in link order before each run), and per node the Winecki-Adams
// link weights as a bit code (bit 0: left link r_m0, 1: right r_p0, 2: lower
// r_0m, 3: upper r_0p; a node is updated iff it has a left or a right link).
template <typename T>
__device__ __forceinline__ void link_U_nodes(const Inst& I, const int (&n)[kCallTiles], int nq) {
    const Geo g = I.g;
    const T* A = (const T*)I.ab[*(volatile int*)&I.st->rhsA];
    C2<T>* U = (C2<T>*)I.U;
    const T dt = gsel<T>(I.dt, I.fdt), sx = dt * GT(g, idx2), sy = dt * GT(g, idy2);
    unsigned cbq[kCallTiles];
    T aa[kCallTiles], ab[kCallTiles];
    // loads of all the thread's nodes first ...
#pragma unroll
    for (int q = 0; q < kCallTiles; ++q) {
        cbq[q] = 0u;
        aa[q] = T(0);
        ab[q] = T(0);
        if (q < nq && n[q] < g.N) {
            const int i = n[q] % g.Nx, j = n[q] / g.Nx;
            cbq[q] = cell_bits(g, I.mt, i, j);
            if (i < g.Nx - 1) aa[q] = A[i + (g.Nx - 1) * j];
            if (j < g.Ny - 1) ab[q] = A[g.Na + i + g.Nx * j];
        }
    }
    // ... then the factors and the stores
#pragma unroll
    for (int q = 0; q < kCallTiles; ++q) {
        if (q >= nq || n[q] >= g.N) continue;
        const int i = n[q] % g.Nx, j = n[q] / g.Nx;
        const unsigned cb = cbq[q];
        const unsigned rm0 = (GL_MM(cb) || GL_MP(cb)) ? 1u : 0u, rp0 = (GL_PM(cb) || GL_PP(cb)) ? 1u : 0u;
        const unsigned r0m = (GL_MM(cb) || GL_PM(cb)) ? 1u : 0u, r0p = (GL_MP(cb) || GL_PP(cb)) ? 1u : 0u;
        I.code[n[q]] = (uint8_t)(rm0 | (rp0 << 1) | (r0m << 2) | (r0p << 3));
        const C2<T> z = cmk<T>(T(0), T(0));
        C2<T> ua = z, ub = z;
        if (i < g.Nx - 1 && rp0) ua = cscale(sx, link_U<T>(GT(g, dx) * aa[q]));
        if (j < g.Ny - 1 && r0p) ub = cscale(sy, link_U<T>(GT(g, dy) * ab[q]));
        if constexpr (sizeof(T) == 4) {
            ((float4*)U)[n[q]] = make_float4(ua.x, ua.y, ub.x, ub.y);
        } else {
            U[2 * n[q]] = ua;
            U[2 * n[q] + 1] = ub;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_link_U(const Inst* __restrict__ insts, const Tile* __restrict__ tiles, int ntiles, int only_solveA) {
    Tile t[kCallTiles];
    const bool same = call_tiles(tiles, ntiles, t);
    auto skip = [&](const Inst& I) {
        // A of a kappa=inf instance does not change, unless fixed vortices add to it
        return only_solveA && !I.solveA && !I.vpi;
    };
    if (same) {
        if (t[0].inst < 0) return;
        const Inst& I = insts[t[0].inst];
        if (skip(I)) return;
        int n[kCallTiles];
        int nq = 0;
#pragma unroll
        for (int q = 0; q < kCallTiles; ++q) {
            n[q] = t[q].n0 + threadIdx.x;
            if (t[q].inst >= 0) nq = q + 1;
        }
        link_U_nodes<T>(I, n, nq);
    } else {
        for (int q = 0; q < kCallTiles; ++q) {
            if (t[q].inst < 0) break;
            const Inst& I = insts[t[q].inst];
            if (skip(I)) continue;
            int n[kCallTiles] = {t[q].n0 + (int)threadIdx.x};
            link_U_nodes<T>(I, n, 1);
        }
    }
}

// Fixed vortices (svirl/solvers/td.py:120-154,204-216,252-325).  Around each psi
// step the reference adds the irregular vector potential to A and subtracts it
// again, and around each A loop it adds A to the irregular potential (used as
// the supercurrent argument) and subtracts the final A; xpy_r / xmy_r run over
// the first N elements of the Nab-long link arrays, and these kernels keep that
// range: thread n handles element n < N.  After the psi loop, psi at the
// phase-lock nodes becomes |psi| (td.h:295-307).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_fv_psi_pre(const Inst* __restrict__ insts, const Tile* __restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const int n = t.n0 + threadIdx.x;
    if (!I.vpi || n >= I.g.N) return;
    T* A = (T*)I.ab[*(volatile const int*)&I.st->rhsA];
    A[n] += ((const T*)I.vpi)[n];
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_fv_psi_post(const Inst* __restrict__ insts, const Tile* __restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const int n = t.n0 + threadIdx.x;
    if (n < I.lock_n) {
        C2<T>* psi = (C2<T>*)I.psi[*(volatile const int*)&I.st->rhs];
        const int m = I.lock[n];
        const C2<T> p = psi[m];
        psi[m] = cmk<T>(hypot(p.x, p.y), T(0));
    }
    if (I.vpi && n < I.g.N) {
        T* A = (T*)I.ab[*(volatile const int*)&I.st->rhsA];
        A[n] -= ((const T*)I.vpi)[n];
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_fv_A(const Inst* __restrict__ insts, const Tile* __restrict__ tiles, int post) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const int n = t.n0 + threadIdx.x;
    if (!I.vpi || !I.solveA || n >= I.g.N) return;
    const T a = ((const T*)I.ab[*(volatile const int*)&I.st->rhsA])[n];
    T* vpi = (T*)I.vpi;
    if (post) vpi[n] -= a;
    else vpi[n] += a;
}

// Start of a Jacobi loop: reset the per-instance loop state and the while
// condition.  which: 0 = psi loop, 1 = A loop; kappa=inf instances have no A loop
// (svirl/solvers/td.py:476).
__global__ void k_loop_begin(const Inst* __restrict__ insts, int ninst, LoopState* loop,
                             cudaGraphConditionalHandle cond, int use_cond, int which) {
    int active = 0;
    for (int q = threadIdx.x; q < ninst; q += blockDim.x) {
        InstState* st = insts[q].st;
        const bool part = which == 0 || insts[q].solveA;
        st->sweep = 0;
        st->done = part ? 0 : 1;
        if (which == 1) st->commitA = 0;
        st->blocks_done = 0u;
        st->res = 0ull;
        for (int l = 0; l < 4; ++l) st->resp[l] = 0ull;
        st->nanlv = 0;
        active += part ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) active += __shfl_down_sync(0xffffffffu, active, o);
    if (threadIdx.x == 0) {
        loop->active = active;
        loop->launches = 0;
        loop->blocks_done = 0u;
        loop->cont = active > 0 ? 1 : 0;
        if (use_cond) cudaGraphSetConditional(cond, active > 0 ? 1u : 0u);
    }
}

// End of a Jacobi loop: advance the Langevin seed of the instances that ran it
// (td.py:204,313); after an A loop no commit is pending any more.
__global__ void k_loop_end(const Inst* __restrict__ insts, int ninst, int which) {
    for (int q = threadIdx.x; q < ninst; q += blockDim.x) {
        if (which == 0 || insts[q].solveA) insts[q].st->rand_t += 1u;
        if (which == 1) insts[q].st->commitA = 0;
    }
}

// After an FP32 A loop: the state buffer holds the offsets delta = A - A^(0) of
// the loop's last sweep (k_A_sweep); A = A^(0) + delta, in place.  A loop that
// stopped on the guard leaves no commit pending and the state at A^(0).
__global__ void __launch_bounds__(kThreads) k_A_commit(const Inst* __restrict__ insts, const Tile* __restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    const Inst& I = insts[t.inst];
    const int c = *(volatile const int*)&I.st->commitA;
    if (c == 0) return;
    const Geo g = I.g;
    const int n = t.n0 + threadIdx.x;
    if (n >= g.N) return;
    const float* base = (const float*)I.ab[c - 1];
    float* A = (float*)I.ab[*(volatile const int*)&I.st->rhsA];
    const int i = n % g.Nx, j = n / g.Nx;
    if (i < g.Nx - 1) {
        const int na = i + (g.Nx - 1) * j;
        A[na] = base[na] + A[na];
    }
    if (j < g.Ny - 1) {
        const int nb = g.Na + i + g.Nx * j;
        A[nb] = base[nb] + A[nb];
    }
}

// End of a time step: count it and decide whether the time loop goes on.
__global__ void k_step_end(const Inst* __restrict__ insts, int ninst, LoopState* loop,
                           cudaGraphConditionalHandle cond, int use_cond) {
    for (int q = threadIdx.x; q < ninst; q += blockDim.x) insts[q].st->steps += 1;
    if (threadIdx.x == 0) {
        int s = loop->step + 1;
        loop->step = s;
        if (use_cond) cudaGraphSetConditional(cond, s < loop->Nt ? 1u : 0u);
    }
}

// After a TD call: move psi and A back into buffer 0 (kCallTiles tiles per CTA,
// all of a thread's loads before its stores).
template <typename T>
__device__ __forceinline__ void canonical_nodes(const Inst& I, const int (&n)[kCallTiles], int nq) {
    const Geo g = I.g;
    const int R = *(volatile int*)&I.st->rhs, RA = *(volatile int*)&I.st->rhsA;
    if (R != 0) {
        const C2<T>* src = (const C2<T>*)I.psi[R];
        C2<T>* dst = (C2<T>*)I.psi[0];
        C2<T> v[kCallTiles];
#pragma unroll
        for (int q = 0; q < kCallTiles; ++q)
            if (q < nq && n[q] < g.N) v[q] = src[n[q]];
#pragma unroll
        for (int q = 0; q < kCallTiles; ++q)
            if (q < nq && n[q] < g.N) dst[n[q]] = v[q];
    }
    if (RA != 0) {
        const T* src = (const T*)I.ab[RA];
        T* dst = (T*)I.ab[0];
        T va[kCallTiles], vb[kCallTiles];
        int la[kCallTiles], lb[kCallTiles];
#pragma unroll
        for (int q = 0; q < kCallTiles; ++q) {
            la[q] = -1;
            lb[q] = -1;
            if (q < nq && n[q] < g.N) {
                const int i = n[q] % g.Nx, j = n[q] / g.Nx;
                if (i < g.Nx - 1) { la[q] = i + (g.Nx - 1) * j; va[q] = src[la[q]]; }
                if (j < g.Ny - 1) { lb[q] = g.Na + i + g.Nx * j; vb[q] = src[lb[q]]; }
            }
        }
#pragma unroll
        for (int q = 0; q < kCallTiles; ++q) {
            if (la[q] >= 0) dst[la[q]] = va[q];
            if (lb[q] >= 0) dst[lb[q]] = vb[q];
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_canonical_copy(const Inst* __restrict__ insts, const Tile* __restrict__ tiles, int ntiles) {
    Tile t[kCallTiles];
    if (call_tiles(tiles, ntiles, t)) {
        if (t[0].inst < 0) return;
        int n[kCallTiles];
        int nq = 0;
#pragma unroll
        for (int q = 0; q < kCallTiles; ++q) {
            n[q] = t[q].n0 + threadIdx.x;
            if (t[q].inst >= 0) nq = q + 1;
        }
        canonical_nodes<T>(insts[t[0].inst], n, nq);
    } else {
        for (int q = 0; q < kCallTiles; ++q) {
            if (t[q].inst < 0) break;
            int n[kCallTiles] = {t[q].n0 + (int)threadIdx.x};
            canonical_nodes<T>(insts[t[q].inst], n, 1);
        }
    }
}

__global__ void k_canonical_reset(const Inst* __restrict__ insts, int ninst) {
    for (int q = threadIdx.x; q < ninst; q += blockDim.x) {
        insts[q].st->rhs = 0;
        insts[q].st->rhsA = 0;
        insts[q].st->commitA = 0;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct TDLaunch {
    const Inst* insts;
    const Tile* tiles;
    const ATile* atiles;
    int natiles;
    const Item* items;
    LoopState* loop;
    int ninst, ntiles, nitems, psi_grid, dtype, strip_rows, psi_kind;
    int psi_cn;       // psi time stepping: 0 backward Euler, 1 Crank-Nicolson, 2 its kernel as written
    bool any_solveA;
    bool any_fv;  // an instance has fixed vortices (irregular potential or phase lock)
};

static void* fv_psi_pre_fn(int dt) { return dt == 8 ? (void*)k_fv_psi_pre<double> : (void*)k_fv_psi_pre<float>; }
static void* fv_psi_post_fn(int dt) { return dt == 8 ? (void*)k_fv_psi_post<double> : (void*)k_fv_psi_post<float>; }
static void* fv_A_fn(int dt) { return dt == 8 ? (void*)k_fv_A<double> : (void*)k_fv_A<float>; }

// The psi sweep kernel of a kind (psi_kind): FP64 and FP32 register strip (the
// default), FP32 bulk-copy ring (selected per handle).
static bool psi_bulk(int kind) { return kind == 5; }
template <int V>
static void* psi_sweep_fn_v(int kind, int rows) {
    if constexpr (V < kNumStripRows) {
        constexpr int R = kStripRowsSet[V];
        if (rows == R)
            return kind == 8 ? (void*)k_psi_sweep<double, R>
                             : (kind == 5 ? (void*)k_psi_sweep_bulk<R> : (void*)k_psi_sweep<float, R>);
        return psi_sweep_fn_v<V + 1>(kind, rows);
    } else {
        return nullptr;
    }
}
// the sweep kernel compiled for strip height `rows` (one of kStripRowsSet), and its CTA size
static void* psi_sweep_fn(int kind, int rows) { return psi_sweep_fn_v<0>(kind, rows); }
static int psi_threads(int kind) { return psi_bulk(kind) ? kBulkThreads : kPsiThreads; }

static cudaError_t launch_psi_sweep(int kind, int rows, int grid, cudaStream_t s, const Inst* insts, const Item* items,
                                    int nitems, LoopState* loop) {
    cudaGraphConditionalHandle none = 0;
    int zero = 0;
    void* a[] = {&insts, &items, &nitems, &loop, &none, &zero};
    return cudaLaunchKernel(psi_sweep_fn(kind, rows), dim3(grid), dim3(psi_threads(kind)), a, 0, s);
}
static void* A_sweep_fn(int dtype) {
    return dtype == 8 ? (void*)k_A_sweep<double> : (void*)k_A_sweep<float>;
}
static void* cn_fn(int dtype) {
    return dtype == 8 ? (void*)k_psi_sweep_cn<double> : (void*)k_psi_sweep_cn<float>;
}
static void* link_fn(int dtype) {
    return dtype == 8 ? (void*)k_link_U<double> : (void*)k_link_U<float>;
}

cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, int ndeps,
                              void* fn, dim3 grid, dim3 block, void** args, unsigned smem_bytes) {
    cudaKernelNodeParams p;
    memset(&p, 0, sizeof(p));
    p.func = fn;
    p.gridDim = grid;
    p.blockDim = block;
    p.sharedMemBytes = smem_bytes;
    p.kernelParams = args;
    p.extra = nullptr;
    return cudaGraphAddKernelNode(node, g, deps, ndeps, &p);
}

cudaError_t add_while(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, int ndeps,
                             cudaGraphConditionalHandle h, cudaGraph_t* body) {
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaError_t e = cudaGraphAddNode(node, g, deps, nullptr, ndeps, &p);
    if (e == cudaSuccess) *body = p.conditional.phGraph_out[0];
    return e;
}

#define GCHK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { err = e_; goto fail; } } while (0)

// Build the whole TD run of all instances as one graph:
//   [fixed vortices: A += A_irr, psi-only mode] -> [tables, all instances] -> WHILE(step < Nt) {
//       [A += A_irr] -> [tables, finite-kappa / fixed-vortex instances]
//       -> loop_begin(psi) -> WHILE(active) { psi sweep } -> loop_end(psi) -> [phase lock, A -= A_irr]
//       -> [A_irr += A] -> loop_begin(A) -> WHILE(active) { A sweep } -> loop_end(A) -> [A_irr -= A]
//       -> step_end }
//   -> canonical copy -> canonical reset
// (bracketed fixed-vortex kernels only when an instance has fixed vortices; in
// psi-only mode A += A_irr runs once before the time loop, as in the reference,
// td.py:216-223).
static cudaError_t build_td_graph(const TDLaunch& L, int eqn, cudaGraphExec_t* exec) {
    cudaError_t err = cudaSuccess;
    cudaGraph_t top = nullptr, obody = nullptr, pbody = nullptr, abody = nullptr;
    cudaGraphConditionalHandle hout, hpsi = 0, hA = 0;
    cudaGraphNode_t n_out = nullptr, n_cc = nullptr, n_cr = nullptr, prev = nullptr, nd;
    const bool do_psi = eqn != 2, do_A = (eqn != 1) && L.any_solveA;
    int zero = 0, one = 1;
    const dim3 gt(L.ntiles), bt(kThreads), g1(1), b1(32);
    Inst const* insts = L.insts;
    Tile const* tiles = L.tiles;
    Item const* items = L.items;
    LoopState* loop = L.loop;
    int ninst = L.ninst, nitems = L.nitems, ntiles = L.ntiles;
    // appends a kernel node after `prev` in graph `g`
    auto chain = [&](cudaGraph_t g, void* fn, dim3 grid, dim3 block, void** a) -> cudaError_t {
        cudaError_t e = add_kernel(g, &nd, prev ? &prev : nullptr, prev ? 1 : 0, fn, grid, block, a);
        if (e == cudaSuccess) prev = nd;
        return e;
    };

    GCHK(cudaGraphCreate(&top, 0));
    GCHK(cudaGraphConditionalHandleCreate(&hout, top, 1, cudaGraphCondAssignDefault));
    if (do_psi && eqn == 1 && L.any_fv) {
        void* a[] = {&insts, &tiles};
        GCHK(chain(top, fv_psi_pre_fn(L.dtype), gt, bt, a));
    }
    if (do_psi) {
        void* a[] = {&insts, &tiles, &ntiles, &zero};
        GCHK(chain(top, link_fn(L.dtype), dim3(call_grid(ntiles)), bt, a));
    }
    GCHK(add_while(top, &n_out, prev ? &prev : nullptr, prev ? 1 : 0, hout, &obody));
    prev = nullptr;
    if (do_psi) {
        GCHK(cudaGraphConditionalHandleCreate(&hpsi, obody, 1, cudaGraphCondAssignDefault));
        if (eqn == 0 && L.any_fv) {
            void* a[] = {&insts, &tiles};
            GCHK(chain(obody, fv_psi_pre_fn(L.dtype), gt, bt, a));
        }
        if (L.any_solveA || L.any_fv) {
            void* a[] = {&insts, &tiles, &ntiles, &one};
            GCHK(chain(obody, link_fn(L.dtype), dim3(call_grid(ntiles)), bt, a));
        }
        {
            void* a[] = {&insts, &ninst, &loop, &hpsi, &one, &zero};
            GCHK(chain(obody, (void*)k_loop_begin, g1, b1, a));
        }
        GCHK(add_while(obody, &nd, &prev, 1, hpsi, &pbody));
        prev = nd;
        {
            cudaGraphNode_t sw;
            if (L.psi_cn) {
                int aw = L.psi_cn == 2 ? 1 : 0;
                void* a[] = {&insts, &tiles, &loop, &hpsi, &one, &aw};
                GCHK(add_kernel(pbody, &sw, nullptr, 0, cn_fn(L.dtype), gt, bt, a));
            } else {
                void* a[] = {&insts, &items, &nitems, &loop, &hpsi, &one};
                GCHK(add_kernel(pbody, &sw, nullptr, 0, psi_sweep_fn(L.psi_kind, L.strip_rows), dim3(L.psi_grid),
                                dim3(psi_threads(L.psi_kind)), a));
            }
        }
        {
            void* a[] = {&insts, &ninst, &zero};
            GCHK(chain(obody, (void*)k_loop_end, g1, b1, a));
        }
        if (L.any_fv) {
            void* a[] = {&insts, &tiles};
            GCHK(chain(obody, fv_psi_post_fn(L.dtype), gt, bt, a));
        }
    }
    if (do_A) {
        GCHK(cudaGraphConditionalHandleCreate(&hA, obody, 1, cudaGraphCondAssignDefault));
        if (L.any_fv) {
            void* a[] = {&insts, &tiles, &zero};
            GCHK(chain(obody, fv_A_fn(L.dtype), gt, bt, a));
        }
        {
            void* a[] = {&insts, &ninst, &loop, &hA, &one, &one};
            GCHK(chain(obody, (void*)k_loop_begin, g1, b1, a));
        }
        GCHK(add_while(obody, &nd, &prev, 1, hA, &abody));
        prev = nd;
        {
            cudaGraphNode_t sw;
            ATile const* atiles = L.atiles;
            void* a[] = {&insts, &atiles, &loop, &hA, &one};
            GCHK(add_kernel(abody, &sw, nullptr, 0, A_sweep_fn(L.dtype), dim3(L.natiles), bt, a));
        }
        if (L.dtype == 4) {
            void* a[] = {&insts, &tiles};
            GCHK(chain(obody, (void*)k_A_commit, gt, bt, a));
        }
        {
            void* a[] = {&insts, &ninst, &one};
            GCHK(chain(obody, (void*)k_loop_end, g1, b1, a));
        }
        if (L.any_fv) {
            void* a[] = {&insts, &tiles, &one};
            GCHK(chain(obody, fv_A_fn(L.dtype), gt, bt, a));
        }
    }
    {
        void* a[] = {&insts, &ninst, &loop, &hout, &one};
        GCHK(chain(obody, (void*)k_step_end, g1, b1, a));
    }
    {
        void* a[] = {&insts, &tiles, &ntiles};
        void* fn = L.dtype == 8 ? (void*)k_canonical_copy<double> : (void*)k_canonical_copy<float>;
        GCHK(add_kernel(top, &n_cc, &n_out, 1, fn, dim3(call_grid(ntiles)), bt, a));
        void* b[] = {&insts, &ninst};
        GCHK(add_kernel(top, &n_cr, &n_cc, 1, (void*)k_canonical_reset, g1, b1, b));
    }
    GCHK(cudaGraphInstantiate(exec, top, 0));
    cudaGraphDestroy(top);
    return cudaSuccess;
fail:
    if (top) cudaGraphDestroy(top);
    *exec = nullptr;
    return err;
}

static void launch_link_U(const TDLaunch& L, int only_solveA, cudaStream_t s) {
    if (L.dtype == 8) k_link_U<double><<<call_grid(L.ntiles), kThreads, 0, s>>>(L.insts, L.tiles, L.ntiles, only_solveA);
    else k_link_U<float><<<call_grid(L.ntiles), kThreads, 0, s>>>(L.insts, L.tiles, L.ntiles, only_solveA);
}

// Host-driven fallback: the same kernels, the loop decided on the host after
// each chunk of sweeps (sweeps of finished instances are no-ops).
static cudaError_t run_host_loop(const TDLaunch& L, int eqn, int Nt, cudaStream_t s) {
    const bool do_psi = eqn != 2, do_A = (eqn != 1) && L.any_solveA;
    const int chunk = 4;
    cudaGraphConditionalHandle none = 0;
    int cont = 1;
    auto fv_psi = [&](bool post) {
        if (L.dtype == 8) {
            if (post) k_fv_psi_post<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
            else k_fv_psi_pre<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
        } else {
            if (post) k_fv_psi_post<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
            else k_fv_psi_pre<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
        }
    };
    auto fv_A = [&](int post) {
        if (L.dtype == 8) k_fv_A<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, post);
        else k_fv_A<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, post);
    };
    if (do_psi && eqn == 1 && L.any_fv) fv_psi(false);
    if (do_psi) launch_link_U(L, 0, s);
    for (int step = 0; step < Nt; ++step) {
        for (int part = 0; part < 2; ++part) {
            if (part == 0 && !do_psi) continue;
            if (part == 1 && !do_A) continue;
            if (part == 0 && eqn == 0 && L.any_fv) fv_psi(false);
            if (part == 0 && (L.any_solveA || L.any_fv)) launch_link_U(L, 1, s);
            if (part == 1 && L.any_fv) fv_A(0);
            k_loop_begin<<<1, 32, 0, s>>>(L.insts, L.ninst, L.loop, none, 0, part);
            for (;;) {
                for (int c = 0; c < chunk; ++c) {
                    if (part == 0 && L.psi_cn) {
                        const int aw = L.psi_cn == 2 ? 1 : 0;
                        if (L.dtype == 8)
                            k_psi_sweep_cn<double><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.loop, none, 0, aw);
                        else
                            k_psi_sweep_cn<float><<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles, L.loop, none, 0, aw);
                    } else if (part == 0) {
                        launch_psi_sweep(L.psi_kind, L.strip_rows, L.psi_grid, s, L.insts, L.items, L.nitems, L.loop);
                    } else {
                        if (L.dtype == 8) k_A_sweep<double><<<L.natiles, kThreads, 0, s>>>(L.insts, L.atiles, L.loop, none, 0);
                        else k_A_sweep<float><<<L.natiles, kThreads, 0, s>>>(L.insts, L.atiles, L.loop, none, 0);
                    }
                }
                cudaError_t e = cudaMemcpyAsync(&cont, &L.loop->cont, sizeof(int), cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) return e;
                e = cudaStreamSynchronize(s);
                if (e != cudaSuccess) return e;
                if (!cont) break;
            }
            if (part == 1 && L.dtype == 4) k_A_commit<<<L.ntiles, kThreads, 0, s>>>(L.insts, L.tiles);
            k_loop_end<<<1, 32, 0, s>>>(L.insts, L.ninst, part);
            if (part == 0 && L.any_fv) fv_psi(true);
            if (part == 1 && L.any_fv) fv_A(1);
        }
        k_step_end<<<1, 32, 0, s>>>(L.insts, L.ninst, L.loop, none, 0);
    }
    if (L.dtype == 8) k_canonical_copy<double><<<call_grid(L.ntiles), kThreads, 0, s>>>(L.insts, L.tiles, L.ntiles);
    else k_canonical_copy<float><<<call_grid(L.ntiles), kThreads, 0, s>>>(L.insts, L.tiles, L.ntiles);
    k_canonical_reset<<<1, 32, 0, s>>>(L.insts, L.ninst);
    return cudaGetLastError();
}

// Prepare one timed sweep: Jacobi sweep index k (k >= 1 reads a psi^(k) buffer
// distinct from the right-hand side, as in a typical sweep), loop not done, and
// the right-hand sides at buffer 0 as at rest (a timed launch that meets the stop
// rule moves them, and the next launch would then write into buffer 0).
__global__ void k_bench_prep(const Inst* __restrict__ insts, int ninst, LoopState* loop, int k) {
    for (int q = threadIdx.x; q < ninst; q += blockDim.x) {
        InstState* st = insts[q].st;
        st->rhs = 0;
        st->rhsA = 0;
        st->sweep = k;
        st->done = 0;
        st->blocks_done = 0u;
        st->res = 0ull;
        for (int l = 0; l < 4; ++l) st->resp[l] = 0ull;
        st->nanlv = 0;
    }
    if (threadIdx.x == 0) {
        loop->active = ninst;
        loop->launches = 0;
        loop->blocks_done = 0u;
        loop->cont = 1;
    }
}

// Per-call counters of every instance back to zero.
// With `loop`, also the time loop's state for a call of Nt steps (written here rather
// than copied from the host, which saves a transfer per call).
__global__ void k_reset_counters(const Inst* __restrict__ insts, int ninst, LoopState* loop, int Nt, int guard) {
    if (loop && blockIdx.x == 0 && threadIdx.x == 0) {
        LoopState ls;
        memset(&ls, 0, sizeof(ls));
        ls.Nt = Nt;
        ls.ninst = ninst;
        ls.guard = guard;
        *loop = ls;
    }
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ninst; q += gridDim.x * blockDim.x) {
        InstState* st = insts[q].st;
        st->nan_seen = 0;
        st->last_sweeps_psi = st->last_sweeps_A = st->max_sweeps_psi = st->max_sweeps_A = 0;
        st->total_sweeps_psi = st->total_sweeps_A = 0;
        st->steps = 0;
    }
}

// The instances' loop states gathered into one array (one copy to the host).
__global__ void k_gather_states(const Inst* __restrict__ insts, int ninst, InstState* out) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ninst; q += gridDim.x * blockDim.x) out[q] = *insts[q].st;
}

int time_sweeps(glgpu_handle* h, int which, int nrep, double* avg_ms) {
    if (nrep < 1 || which < 0 || which > 1 || !avg_ms) return set_error(h, GLGPU_E_ARG, "time_sweeps: bad arguments");
    const bool solveA = h->p.kappa > 0.0 && !std::isinf(h->p.kappa);
    if (which == 1 && !solveA) return set_error(h, GLGPU_E_ARG, "time_sweeps: A sweeps need a finite kappa");
    const size_t flush_bytes = (size_t)256 << 20;  // > 129 MB of L2
    if (!h->flush && cudaMalloc(&h->flush, flush_bytes) != cudaSuccess) return set_error(h, GLGPU_E_OOM, "time_sweeps: flush buffer");
    h->inst_h.dt = h->inst_h.dt > 0.0 ? h->inst_h.dt : 0.1;
    h->inst_h.fdt = (float)h->inst_h.dt;
    cudaError_t e = cudaMemcpyAsync(h->inst, &h->inst_h, sizeof(Inst), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "time_sweeps");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaGraphConditionalHandle none = 0;
    if (h->dtype == 8) k_link_U<double><<<call_grid(h->ntiles), kThreads, 0, h->stream>>>(h->inst, h->tiles, h->ntiles, 0);
    else k_link_U<float><<<call_grid(h->ntiles), kThreads, 0, h->stream>>>(h->inst, h->tiles, h->ntiles, 0);
    double total = 0.0;
    // A sweeps come in pairs (sweep 0 computes the links' fixed parts, sweep 1 reuses
    // them), so an A repetition times both and the average is over sweeps
    const int per_rep = which == 0 ? 1 : 2;
    for (int r = 0; r < nrep && e == cudaSuccess; ++r) {
        cudaMemsetAsync(h->flush, r & 0xff, flush_bytes, h->stream);
        for (int q = 0; q < per_rep && e == cudaSuccess; ++q) {
            k_bench_prep<<<1, 32, 0, h->stream>>>(h->inst, 1, h->loop, which == 0 ? 1 : q);
            cudaEventRecord(e0, h->stream);
            if (which == 0) {
                launch_psi_sweep(psi_kind(h->dtype, h->psi_select), h->strip_rows, h->psi_grid, h->stream, h->inst, h->items,
                                 h->nitems, h->loop);
            } else {
                if (h->dtype == 8) k_A_sweep<double><<<h->natiles, kThreads, 0, h->stream>>>(h->inst, h->atiles, h->loop, none, 0);
                else k_A_sweep<float><<<h->natiles, kThreads, 0, h->stream>>>(h->inst, h->atiles, h->loop, none, 0);
            }
            cudaEventRecord(e1, h->stream);
            e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            total += ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // leave the loop state as a finished loop; the state at rest (buffer 0) was not written
    k_canonical_reset<<<1, 32, 0, h->stream>>>(h->inst, 1);
    LoopState hl;
    memset(&hl, 0, sizeof(hl));
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hl, h->loop, sizeof(hl), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "time_sweeps");
    if (hl.err & kErrCopyWait) return set_error(h, GLGPU_E_TIMEOUT, "time_sweeps: psi sweep: a bulk-copy wait ran out");
    *avg_ms = total / (nrep * per_rep);
    return GLGPU_OK;
}

// CTAs of the persistent psi sweep (nitems: length of the item table): one warp
// per item (register-strip kernel) or one CTA per group of kPsiGroup items
// (bulk-copy kernel), up to all SMs at full occupancy.
int psi_sweep_grid(int kind, int rows, int nitems) {
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* fn = psi_sweep_fn(kind, rows);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, psi_threads(kind), 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int need = psi_bulk(kind) ? nitems / kPsiGroup : (nitems + kPsiWarps - 1) / kPsiWarps;
    const int full = sms * per_sm;
    return need < full ? (need > 0 ? need : 1) : full;
}

// Strip height for a set of instances (a handle or a batch), from a model of
// the persistent sweep: warps take items round-robin, so a launch lasts as long
// as the warp with the most items, ceil(items / warps), and an item of R rows
// costs about 3R + 6 row-sweeps (sweep l of the kFuse = 3 fused sweeps covers
// R + 2(3 - l) rows).  Measured on 2049^2 (FP32, us per node-sweep): R = 8: 38.1,
// 12: 34.7, 14: 33.5, 17: 32.2, 18: 32.7; the model ranks them the same way.
int choose_strip_rows(int dtype, const Geo* const* geos, int n) {
    int best = kStripRowsSet[0];
    long long best_cost = -1;
    for (int v = 0; v < kNumStripRows; ++v) {
        const int R = kStripRowsSet[v];
        long long table = 0;
        for (int q = 0; q < n; ++q) table += strip_table_len(geos[q]->Nx, geos[q]->Ny, R);
        // work units: groups of kPsiGroup items per CTA (bulk-copy kernel) or items per warp
        const int kind = psi_kind(dtype, 0);
        const bool bulk = psi_bulk(kind);
        const long long units = bulk ? table / kPsiGroup : table;
        const long long slots = (long long)psi_sweep_grid(kind, R, (int)table) * (bulk ? 1 : kPsiWarps);
        const long long cost = (units + slots - 1) / slots * (3LL * R + 2LL * kFuse);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = R;
        }
    }
    return best;
}

// Items of one instance, row-block major (concurrently running warps share halo
// rows in L2); each band's strips padded to a multiple of kPsiGroup with empty items.
std::vector<Item> make_items(const Geo& g, int inst, int rows) {
    std::vector<Item> items;
    const int nstrips = (g.Nx + kStripCols - 1) / kStripCols, nrows = (g.Ny + rows - 1) / rows;
    const int padded = (nstrips + kPsiGroup - 1) / kPsiGroup * kPsiGroup;
    items.reserve((size_t)padded * nrows);
    for (int r = 0; r < nrows; ++r)
        for (int s = 0; s < padded; ++s)
            items.push_back(s < nstrips ? Item{inst, kStripCols * s, rows * r, 0} : Item{-1, 0, 0, 0});
    return items;
}

struct TDOutcome {
    cudaError_t err;
    int used_graph, loop_err, steps;
    float ms;
    long long launches;
};

// One TD call over the instances of L: per-call counters reset, the graph (built
// once per eqn mode and kappa mix) or the host-driven loop, then the instances'
// loop states gathered to the host.
// gather_host and hl: pinned host memory (the call's last copies are asynchronous)
static TDOutcome td_core(cudaStream_t s, const TDLaunch& L, int Nt, int eqn, cudaGraphExec_t* execs, bool* graph_failed,
                         bool use_graphs, int guard, bool timed, InstState* gather_dev, InstState* gather_host,
                         LoopState* hl_pinned) {
    TDOutcome o = {cudaSuccess, 0, 0, 0, 0.f, 0};
    k_reset_counters<<<(L.ninst + 127) / 128, 128, 0, s>>>(L.insts, L.ninst, Nt > 0 ? L.loop : nullptr, Nt,
                                                           guard > 0 ? guard : kLoopGuard);
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (timed) {
        cudaEventCreate(&ev0);
        cudaEventCreate(&ev1);
    }
    LoopState& hl = *hl_pinned;
    memset(&hl, 0, sizeof(hl));
    if (Nt > 0) {
        const int slot = eqn * 4 + (L.any_solveA ? 2 : 0) + (L.any_fv ? 1 : 0);
        if (use_graphs && !*graph_failed) {
            if (execs[slot] == nullptr) {
                if (build_td_graph(L, eqn, &execs[slot]) != cudaSuccess) {
                    *graph_failed = true;
                    cudaGetLastError();
                }
            }
            if (execs[slot] != nullptr) {
                if (ev0) cudaEventRecord(ev0, s);
                o.err = cudaGraphLaunch(execs[slot], s);
                if (o.err != cudaSuccess) return o;
                o.used_graph = 1;
            }
        }
        if (!o.used_graph) {
            if (ev0) cudaEventRecord(ev0, s);
            o.err = run_host_loop(L, eqn, Nt, s);
            if (o.err != cudaSuccess) return o;
        }
        if (ev1) cudaEventRecord(ev1, s);
    }
    k_gather_states<<<(L.ninst + 127) / 128, 128, 0, s>>>(L.insts, L.ninst, gather_dev);
    o.err = cudaMemcpyAsync(gather_host, gather_dev, sizeof(InstState) * (size_t)L.ninst, cudaMemcpyDeviceToHost, s);
    if (o.err == cudaSuccess) o.err = cudaMemcpyAsync(hl_pinned, L.loop, sizeof(hl), cudaMemcpyDeviceToHost, s);
    if (o.err == cudaSuccess) o.err = cudaStreamSynchronize(s);
    if (ev0) {
        if (o.err == cudaSuccess && Nt > 0) cudaEventElapsedTime(&o.ms, ev0, ev1);
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
    }
    o.loop_err = Nt > 0 ? hl.err : 0;
    o.steps = Nt > 0 ? hl.step : 0;
    o.launches = Nt > 0 ? hl.total_launches : 0;
    return o;
}

static void fill_stats(glgpu_td_stats* stats, const InstState* hs, int n, const TDOutcome& o) {
    if (!stats) return;
    memset(stats, 0, sizeof(*stats));
    stats->steps = o.steps;
    stats->used_graph = o.used_graph;
    stats->sweep_launches = o.launches;
    for (int q = 0; q < n; ++q) {
        const InstState& s = hs[q];
        if (s.max_sweeps_psi > stats->max_sweeps_psi) stats->max_sweeps_psi = s.max_sweeps_psi;
        if (s.max_sweeps_A > stats->max_sweeps_A) stats->max_sweeps_A = s.max_sweeps_A;
        stats->last_sweeps_psi = s.last_sweeps_psi;
        stats->last_sweeps_A = s.last_sweeps_A;
        stats->nan_seen |= s.nan_seen;
        stats->total_sweeps_psi += s.total_sweeps_psi;
        stats->total_sweeps_A += s.total_sweeps_A;
        stats->rand_t = s.rand_t;
    }
}

int td_run(glgpu_handle* h, double dt, int Nt, int eqn, glgpu_td_stats* stats, double* elapsed_ms) {
    if (eqn < 0 || eqn > 2 || Nt < 0) return set_error(h, GLGPU_E_ARG, "glgpu_td: bad eqn or Nt");
    // dt of the order-parameter iterator; the A kernel also receives it (td.py:278)
    h->inst_h.dt = dt;
    h->inst_h.fdt = (float)dt;
    // pinned staging: the descriptor upload and the statistics download of a call are
    // asynchronous copies (the stream is synchronised before td_core returns)
    PinStage* ps = (PinStage*)h->pin;
    ps->inst = h->inst_h;
    cudaError_t e = cudaMemcpyAsync(h->inst, &ps->inst, sizeof(Inst), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return cuda_check(h, e, "td: write descriptor");
    TDLaunch L;
    L.insts = h->inst; L.tiles = h->tiles; L.items = h->items; L.loop = h->loop;
    L.atiles = h->atiles; L.natiles = h->natiles;
    L.ninst = 1; L.ntiles = h->ntiles; L.nitems = h->nitems; L.psi_grid = h->psi_grid; L.dtype = h->dtype;
    L.strip_rows = h->strip_rows;
    L.psi_kind = psi_kind(h->dtype, h->psi_select);
    L.psi_cn = h->psi_scheme;
    L.any_solveA = h->inst_h.solveA != 0;
    L.any_fv = h->vpi != nullptr || h->lock_n > 0;
    TDOutcome o = td_core(h->stream, L, Nt, eqn, h->td_exec, &h->td_graph_failed, h->use_graphs, h->loop_guard,
                          elapsed_ms != nullptr,
                          h->st_gather, &ps->st, &ps->loop);
    const InstState hs = ps->st;
    if (o.err != cudaSuccess) return cuda_check(h, o.err, "td");
    if (elapsed_ms) *elapsed_ms = o.ms;
    h->p.rand_t = hs.rand_t;
    fill_stats(stats, &hs, 1, o);
    if (o.loop_err & kErrLoopGuard) return set_error(h, GLGPU_E_TIMEOUT, "td: Jacobi loop guard reached");
    if (o.loop_err & kErrCopyWait) return set_error(h, GLGPU_E_TIMEOUT, "td: psi sweep: a bulk-copy wait ran out");
    if (hs.nan_seen) return set_error(h, GLGPU_E_NAN, "td: NaN residual (the state was updated as the reference does)");
    return GLGPU_OK;
}

int batch_td(glgpu_batch* b, double dt, int Nt, int eqn, glgpu_td_stats* stats, double* elapsed_ms) {
    if (eqn < 0 || eqn > 2 || Nt < 0) return batch_error(b, GLGPU_E_ARG, "batch_td: bad eqn or Nt");
    std::vector<Inst> insts(b->ninst);
    bool any_solveA = false, any_fv = false;
    for (int q = 0; q < b->ninst; ++q)
        if (b->hs[q]->psi_scheme != 0)
            return batch_error(b, GLGPU_E_ARG, "batch_td: Crank-Nicolson instances run on their own handle");
    for (int q = 0; q < b->ninst; ++q) {
        glgpu_handle* h = b->hs[q];
        cudaStreamSynchronize(h->stream);
        h->inst_h.dt = dt;
        h->inst_h.fdt = (float)dt;
        insts[q] = h->inst_h;
        insts[q].nitems = b->inst_items[q];  // at the batch's strip height
        any_solveA = any_solveA || h->inst_h.solveA != 0;
        any_fv = any_fv || h->vpi != nullptr || h->lock_n > 0;
    }
    memcpy(b->insts_pin, insts.data(), sizeof(Inst) * insts.size());
    cudaError_t e = cudaMemcpyAsync(b->insts, b->insts_pin, sizeof(Inst) * insts.size(), cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return batch_error(b, GLGPU_E_CUDA, std::string("batch_td: ") + cudaGetErrorString(e));
    TDLaunch L;
    L.insts = b->insts; L.tiles = b->tiles; L.items = b->items; L.loop = b->loop;
    L.atiles = b->atiles; L.natiles = b->natiles;
    L.ninst = b->ninst; L.ntiles = b->ntiles; L.nitems = b->nitems; L.psi_grid = b->psi_grid; L.dtype = b->dtype;
    L.strip_rows = b->strip_rows;
    L.psi_kind = psi_kind(b->dtype, 0);
    L.psi_cn = 0;
    L.any_solveA = any_solveA;
    L.any_fv = any_fv;
    TDOutcome o = td_core(b->stream, L, Nt, eqn, b->td_exec, &b->td_graph_failed, b->use_graphs, b->loop_guard,
                          elapsed_ms != nullptr,
                          b->gather, b->gather_pin, b->loop_pin);
    if (o.err == cudaSuccess) memcpy(b->gather_h.data(), b->gather_pin, sizeof(InstState) * (size_t)b->ninst);
    if (o.err != cudaSuccess) return batch_error(b, GLGPU_E_CUDA, std::string("batch_td: ") + cudaGetErrorString(o.err));
    if (elapsed_ms) *elapsed_ms = o.ms;
    int nan = 0;
    for (int q = 0; q < b->ninst; ++q) {
        b->hs[q]->p.rand_t = b->gather_h[q].rand_t;
        nan |= b->gather_h[q].nan_seen;
    }
    fill_stats(stats, b->gather_h.data(), b->ninst, o);
    if (o.loop_err & kErrLoopGuard) return batch_error(b, GLGPU_E_TIMEOUT, "batch_td: Jacobi loop guard reached");
    if (o.loop_err & kErrCopyWait) return batch_error(b, GLGPU_E_TIMEOUT, "batch_td: psi sweep: a bulk-copy wait ran out");
    if (nan) return batch_error(b, GLGPU_E_NAN, "batch_td: NaN residual in at least one instance");
    return GLGPU_OK;
}

}  // namespace glgpu
