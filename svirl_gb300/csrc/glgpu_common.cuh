// Shared device-side definitions of the GB300 GL solver (complex helpers, grid
// geometry, cell flags, residual stop rule, FP64 block reductions).
//
// Layouts are the reference's (svirl/cuda/*.h): order parameter psi complex,
// n = i + Nx*j; vector potential one real array [a | b] with
// a[i + (Nx-1)*j] (x links) and b[Na + i + Nx*j] (y links); material tiling one
// byte per cell i + (Nx-1)*j, NULL = whole domain superconducting.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace glgpu {

constexpr int kThreads = 256;      // threads per CTA for all node kernels
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSweeps = 1024;   // Jacobi cap per time step (svirl/solvers/td.py:164,274)
constexpr int kLoopGuard = kMaxSweeps + 64;

// ---------------------------------------------------------------------------
// complex numbers as float2 / double2
// ---------------------------------------------------------------------------
template <typename T> struct C2T;
template <> struct C2T<float> { using type = float2; };
template <> struct C2T<double> { using type = double2; };
template <typename T> using C2 = typename C2T<T>::type;

template <typename T> __device__ __forceinline__ C2<T> cmk(T re, T im) { C2<T> z; z.x = re; z.y = im; return z; }
#define GLGPU_COMPLEX_OPS(V, S)                                                                                 \
    __device__ __forceinline__ V cadd(V a, V b) { V z; z.x = a.x + b.x; z.y = a.y + b.y; return z; }            \
    __device__ __forceinline__ V csub(V a, V b) { V z; z.x = a.x - b.x; z.y = a.y - b.y; return z; }            \
    __device__ __forceinline__ V cmul(V a, V b) { V z; z.x = a.x * b.x - a.y * b.y; z.y = a.x * b.y + a.y * b.x; return z; } \
    __device__ __forceinline__ V cconj(V a) { V z; z.x = a.x; z.y = -a.y; return z; }                            \
    __device__ __forceinline__ V cscale(S s, V a) { V z; z.x = s * a.x; z.y = s * a.y; return z; }              \
    __device__ __forceinline__ S cabs2(V a) { return a.x * a.x + a.y * a.y; }
GLGPU_COMPLEX_OPS(float2, float)
GLGPU_COMPLEX_OPS(double2, double)
#undef GLGPU_COMPLEX_OPS

__device__ __forceinline__ void sincos_t(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_t(double x, double* s, double* c) { sincos(x, s, c); }

// Link factor U(ph) = exp(-i ph) (svirl/cuda/common.h:28-33).
template <typename T> __device__ __forceinline__ C2<T> link_U(T ph) {
    T s, c;
    sincos_t(ph, &s, &c);
    return cmk<T>(c, -s);
}

// Im(conj(psi0) U(ph) psi1) (svirl/cuda/common.h:66-73).
// a * b rounded once, never fused into a neighbouring add
__device__ __forceinline__ float mul_rn_t(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn_t(double a, double b) { return __dmul_rn(a, b); }
template <typename T> __device__ __forceinline__ T mul_rn(T a, T b) { return mul_rn_t(a, b); }

template <typename T> __device__ __forceinline__ T js_of(C2<T> p0, T ph, C2<T> p1) {
    T s, c;
    sincos_t(ph, &s, &c);
    return (p0.x * p1.y - p0.y * p1.x) * c - (p0.x * p1.x + p0.y * p1.y) * s;
}

// |psi1 U(ph) - psi0|^2 (svirl/cuda/observables.h:238-247).
template <typename T> __device__ __forceinline__ T g_grad(C2<T> p0, T ph, C2<T> p1) {
    T s, c;
    sincos_t(ph, &s, &c);
    T re = p1.x * c + p1.y * s - p0.x;
    T im = p1.y * c - p1.x * s - p0.y;
    return re * re + im * im;
}

// psi1 U(ph) - psi0 (svirl/cuda/cg.h:304-311), with (s, c) = sincos(ph) given.
template <typename T> __device__ __forceinline__ C2<T> grad_c_sc(C2<T> p0, T s, T c, C2<T> p1) {
    return cmk<T>(p1.x * c + p1.y * s - p0.x, p1.y * c - p1.x * s - p0.y);
}

// ---------------------------------------------------------------------------
// Langevin random numbers (svirl/cuda/common.h:36-63)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t rand_hash(uint32_t s) {
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}
// 2^-32 * hash: the scale is a power of two, so the product in T is exact and
// equals the reference's double product rounded to T.
template <typename T> __device__ __forceinline__ T rand_1(uint32_t n, uint32_t t) {
    return T(rand_hash(71u * n + 9887u * t)) * T(2.3283064365386962890625e-10);
}
template <typename T> __device__ __forceinline__ T rand_2(uint32_t n, uint32_t t) {
    return T(rand_hash(73u * n + 9901u * t + 1u)) * T(2.3283064365386962890625e-10);
}

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------
// Grid geometry with its derived constants precomputed on the host in double
// and rounded once to float (as the reference bakes 1.0/(dx*dx) etc. into its
// kernels at compile time): FP32 kernels then execute no FP64 instruction,
// which matters on GB300 where the FP64 pipe is a small fraction of FP32.
struct Geo {
    int Nx, Ny, Na, N, Nab, Nxc, Nyc;
    double dx, dy, idx, idy, idx2, idy2, idxy, dxdy;
    float fdx, fdy, fidx, fidy, fidx2, fidy2, fidxy, fdxdy;
};

__host__ __device__ inline Geo make_geo(int Nx, int Ny, double dx, double dy) {
    Geo g;
    g.Nx = Nx; g.Ny = Ny; g.Na = (Nx - 1) * Ny; g.N = Nx * Ny;
    g.Nab = g.Na + Nx * (Ny - 1); g.Nxc = Nx - 1; g.Nyc = Ny - 1;
    g.dx = dx; g.dy = dy;
    g.idx = 1.0 / dx; g.idy = 1.0 / dy;
    g.idx2 = 1.0 / (dx * dx); g.idy2 = 1.0 / (dy * dy); g.idxy = 1.0 / (dx * dy);
    g.dxdy = dx * dy;
    g.fdx = (float)dx; g.fdy = (float)dy; g.fidx = (float)g.idx; g.fidy = (float)g.idy;
    g.fidx2 = (float)g.idx2; g.fidy2 = (float)g.idy2; g.fidxy = (float)g.idxy; g.fdxdy = (float)g.dxdy;
    return g;
}

// The T-precision copy of a constant stored in both precisions.
template <typename T> __host__ __device__ __forceinline__ T gsel(double d, float f);
template <> __host__ __device__ __forceinline__ float gsel<float>(double, float f) { return f; }
template <> __host__ __device__ __forceinline__ double gsel<double>(double d, float) { return d; }
#define GT(g, name) gsel<T>((g).name, (g).f##name)

// Cells around node (i, j): bit 0 = (i-1,j-1) "mm", 1 = (i-1,j) "mp",
// 2 = (i,j-1) "pm", 3 = (i,j) "pp"; a bit is set when the cell exists and is in
// material (svirl/cuda/td.h:129-138).
__device__ __forceinline__ unsigned cell_bits(const Geo& g, const uint8_t* __restrict__ mt, int i, int j) {
    bool mm = (i > 0) && (j > 0);
    bool mp = (i > 0) && (j + 1 < g.Ny);
    bool pm = (i + 1 < g.Nx) && (j > 0);
    bool pp = (i + 1 < g.Nx) && (j + 1 < g.Ny);
    if (mt != nullptr) {
        if (mm) mm = mt[(i - 1) + g.Nxc * (j - 1)] != 0;
        if (mp) mp = mt[(i - 1) + g.Nxc * j] != 0;
        if (pm) pm = mt[i + g.Nxc * (j - 1)] != 0;
        if (pp) pp = mt[i + g.Nxc * j] != 0;
    }
    return (mm ? 1u : 0u) | (mp ? 2u : 0u) | (pm ? 4u : 0u) | (pp ? 8u : 0u);
}
#define GL_MM(b) (((b) & 1u) != 0)
#define GL_MP(b) (((b) & 2u) != 0)
#define GL_PM(b) (((b) & 4u) != 0)
#define GL_PP(b) (((b) & 8u) != 0)

// ---------------------------------------------------------------------------
// Jacobi stop rule (svirl/cuda/td.h:205-213, svirl/solvers/td.py:198-202):
// per node code = int32(min(1e4*r/eps, 1e8)) in the kernel's precision, stop
// when 1e-4*max(code) < 1, i.e. when the code of the largest residual is below
// 10000 (the code is monotone in r, so the max residual decides).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool jacobi_converged(float r, double stop) {
    float x = (float)((1.0e4 * (double)r) / (double)(float)stop);
    if (x > 1.0e8) x = 1.0e8f;
    return (int)x < 10000;
}
__device__ __forceinline__ bool jacobi_converged(double r, double stop) {
    double x = (1.0e4 * r) / stop;
    if (x > 1.0e8) x = 1.0e8;
    return (int)x < 10000;
}

// Residuals are non-negative, so their IEEE bit patterns order like the values.
__device__ __forceinline__ unsigned long long res_bits(float r) { return (unsigned long long)__float_as_uint(r); }
__device__ __forceinline__ unsigned long long res_bits(double r) { return (unsigned long long)__double_as_longlong(r); }
template <typename T> __device__ __forceinline__ T res_from_bits(unsigned long long b);
template <> __device__ __forceinline__ float res_from_bits<float>(unsigned long long b) { return __uint_as_float((unsigned)b); }
template <> __device__ __forceinline__ double res_from_bits<double>(unsigned long long b) { return __longlong_as_double((long long)b); }

// ---------------------------------------------------------------------------
// block reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ int flat_tid() { return threadIdx.x + blockDim.x * threadIdx.y; }

template <typename T> __device__ __forceinline__ T warp_max(T v) {
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_down_sync(0xffffffffu, v, o);
        v = v > w ? v : w;
    }
    return v;
}

// Sum NV doubles over the CTA; thread 0 gets the totals.  Fixed order: the
// result is deterministic for a given launch shape.
template <int NV> __device__ __forceinline__ void block_sum(double (&v)[NV]) {
    __shared__ double sm[kWarps][NV];
    const int tid = flat_tid(), lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sm[w][k] = v[k];
    __syncthreads();
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (int q = 0; q < kWarps; ++q) s += sm[q][k];
            v[k] = s;
        }
    }
}

// Error-free sum (Knuth's two-sum): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Sum NV per-thread float values over the CTA into doubles (thread 0).  Every
// partial is carried as a float pair hi + lo, the rounding error of each
// addition kept by two_sum (double-float arithmetic, close to FP64 accuracy):
// a 5-level shuffle tree per warp, then thread k adds the warps' pairs of
// component k in warp order and widens once to double.  GB300 issues an FP64
// instruction at a small fraction of the FP32 rate whatever the number of
// active lanes, so the reduction keeps FP64 to three instructions per CTA.
// Fixed order: deterministic.
template <int NV> __device__ __forceinline__ void block_sum(const float (&v)[NV], double (&out)[NV]) {
    static_assert(NV <= kThreads, "one thread per component");
    __shared__ float sh[kWarps][NV], sl[kWarps][NV];
    __shared__ double so[NV];
    const int tid = flat_tid(), lane = tid & 31, w = tid >> 5;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        float hi = v[k], lo = 0.f;
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
            float sum, err;
            two_sum(hi, oh, sum, err);
            hi = sum;
            lo = lo + (ol + err);
        }
        if (lane == 0) {
            sh[w][k] = hi;
            sl[w][k] = lo;
        }
    }
    __syncthreads();
    if (tid < NV) {
        float hi = sh[0][tid], lo = sl[0][tid];
#pragma unroll
        for (int q = 1; q < kWarps; ++q) {
            float sum, err;
            two_sum(hi, sh[q][tid], sum, err);
            hi = sum;
            lo = lo + (sl[q][tid] + err);
        }
        so[tid] = (double)hi + (double)lo;
    }
    __syncthreads();
    if (tid == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = so[k];
}
template <int NV> __device__ __forceinline__ void block_sum(const double (&v)[NV], double (&out)[NV]) {
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = v[k];
    block_sum<NV>(out);
}

// Grid-wide FP64 vector sum in one launch: every CTA stores its partials, the
// last CTA to finish (ticket counter) adds the partials in block order and
// writes NV results to out[] (scaled by `scale`).  `counter` must be 0 on entry
// and is left 0.  Per-thread inputs in the kernel's precision T.
template <typename T, int NV>
__device__ void grid_sum_finish(const T (&vin)[NV], double* __restrict__ partials, unsigned* counter,
                                double* __restrict__ out, double scale) {
    __shared__ bool last;
    double v[NV];
    block_sum<NV>(vin, v);
    const int tid = flat_tid();
    const int nblk = gridDim.x * gridDim.y;
    const int bid = blockIdx.x + gridDim.x * blockIdx.y;
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) partials[(size_t)bid * NV + k] = v[k];
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        last = (t == (unsigned)nblk - 1u);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int b = tid; b < nblk; b += blockDim.x * blockDim.y)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += ((volatile double*)partials)[(size_t)b * NV + k];
    block_sum<NV>(acc);
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k] = acc[k] * scale;
        *counter = 0u;
    }
}

}  // namespace glgpu
