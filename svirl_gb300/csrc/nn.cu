// Kernels of the learned CG warm start: the fallback weight gradient of the 3x3
// convolution as an implicit GEMM on mma.sync (bf16 -> f32), pooling/upsampling,
// a weighted squared-error loss and Adam.  The forward convolution, its data
// gradient and, for channel counts that are multiples of 64, the weight gradient
// run on tcgen05 (nn_tc.cu).  No counterpart in the reference (its only minimiser
// is the CG of svirl/solvers/cg.py).
//
// Fallback weight gradient: M = cout, N = 9 cin, K = pixels; A = dy^T (with the
// layer's ReLU derivative applied while gathering), B = the input shifted by the
// tap.  A CTA of 4 warps computes a 64 x 64 tile, each warp 32 x 32 (2 x 4
// mma.m16n8k16), over K chunks of 32 staged in shared memory with register
// prefetch of the next chunk; the pixel range is split over CTAs (split-K) and
// the partial sums are reduced in a fixed order (deterministic).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "../../include/glgpu.h"
#include "../../include/glgpu_nn.h"

namespace glnn {

typedef __nv_bfloat16 bf16;

constexpr int BM = 64, BN = 64, BK = 32, NT = 128;
constexpr int SP = BK + 8;  // row stride of a [rows][k] tile (80 B: ldmatrix rows hit distinct banks)
constexpr int TP = 64 + 8;  // row stride of a [k][rows] tile

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t a, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t a, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One BK chunk of the warp-tiled product.  TA: A staged as [BK][TP] (k rows, m
// contiguous) instead of [BM][SP]; TB likewise for B with n.
template <bool TA, bool TB>
__device__ __forceinline__ void mma_chunk(const bf16* As, const bf16* Bs, float (&acc)[2][4][4], int wm, int wn,
                                          int lane) {
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
        uint32_t a[2][4], b[4][2];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const int mb = wm * 32 + mt * 16;
            if (!TA) {
                const bf16* p = As + (mb + (lane & 15)) * SP + ks + (lane >> 4) * 8;
                ldsm_x4(saddr(p), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
            } else {
                const bf16* p = As + (ks + (lane & 7) + (lane >> 4) * 8) * TP + mb + ((lane >> 3) & 1) * 8;
                ldsm_x4_t(saddr(p), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
            }
        }
#pragma unroll
        for (int np = 0; np < 2; ++np) {
            const int nb = wn * 32 + np * 16;
            uint32_t r0, r1, r2, r3;
            if (!TB) {
                const bf16* p = Bs + (nb + (lane & 7) + (lane >> 4) * 8) * SP + ks + ((lane >> 3) & 1) * 8;
                ldsm_x4(saddr(p), r0, r1, r2, r3);
            } else {
                const bf16* p = Bs + (ks + (lane & 7) + ((lane >> 3) & 1) * 8) * TP + nb + (lane >> 4) * 8;
                ldsm_x4_t(saddr(p), r0, r1, r2, r3);
            }
            b[2 * np][0] = r0;
            b[2 * np][1] = r1;
            b[2 * np + 1][0] = r2;
            b[2 * np + 1][1] = r3;
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], a[mt], b[nt][0], b[nt][1]);
    }
}

// dy * (y > 0) on two packed bf16 values (y > 0: sign clear and not zero).
__device__ __forceinline__ uint32_t relu_mask2(uint32_t d, uint32_t y) {
    const uint32_t lo = ((y & 0xffffu) - 1u) < 0x7fffu ? 0x0000ffffu : 0u;
    const uint32_t hi = ((y >> 16) - 1u) < 0x7fffu ? 0xffff0000u : 0u;
    return d & (lo | hi);
}
__device__ __forceinline__ uint4 relu_mask8(uint4 d, uint4 y) {
    return make_uint4(relu_mask2(d.x, y.x), relu_mask2(d.y, y.y), relu_mask2(d.z, y.z), relu_mask2(d.w, y.w));
}

struct Pix {
    int n, y, x;
    bool ok;
};
__device__ __forceinline__ Pix pix_of(int p, int P, int H, int W) {
    Pix q;
    q.ok = p < P;
    const int pp = q.ok ? p : 0;
    q.x = pp % W;
    const int t = pp / W;
    q.y = t % H;
    q.n = t / H;
    return q;
}

// 8 channels (ci..ci+7) of pixel (n, sy, sx) of the concatenation [x1 | x2].
__device__ __forceinline__ uint4 load_cat8(const bf16* x1, int C1, const bf16* x2, int C2, int n, int sy, int sx,
                                           int H, int W, int ci) {
    const size_t q = ((size_t)n * H + sy) * W + sx;
    return ci < C1 ? *(const uint4*)(x1 + q * C1 + ci) : *(const uint4*)(x2 + q * C2 + (ci - C1));
}

// ---------------------------------------------------------------------------
// weight gradient: dW[co][tap][ci] = sum_p dy'[p][co] x[p + off(tap)][ci],
// split over pixel ranges (blockIdx.z); partial tiles go to ws[z][co][n].
// ---------------------------------------------------------------------------
template <int RELU>
__global__ void __launch_bounds__(NT)
k_conv_bwd_weight(const bf16* __restrict__ dy, const bf16* __restrict__ yv, const bf16* __restrict__ x1, int C1,
                  const bf16* __restrict__ x2, int C2, float* __restrict__ ws, int NB, int H, int W, int Cout,
                  int chunk) {
    __shared__ __align__(16) bf16 At[BK * TP];
    __shared__ __align__(16) bf16 Bt[BK * TP];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, wm = warp >> 1, wn = warp & 1;
    const int Cin = C1 + C2, N9 = 9 * Cin, P = NB * H * W;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int pbeg = blockIdx.z * chunk, pend = min(P, pbeg + chunk);
    uint4 ra[2], rb[2];
    const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
    auto load = [&](int pk) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int v = tid + i * NT, kr = v >> 3, c8 = (v & 7) * 8;
            const int p = pk + kr;
            uint4 a = z4, b = z4;
            if (p < pend) {
                const int co = m0 + c8;
                if (co < Cout) {
                    const size_t q = (size_t)p * Cout + co;
                    a = *(const uint4*)(dy + q);
                    if (RELU) a = relu_mask8(a, *(const uint4*)(yv + q));
                }
                const int n = n0 + c8;
                if (n < N9) {
                    const int tap = n / Cin, ci = n - tap * Cin;
                    const Pix px = pix_of(p, P, H, W);
                    const int sy = px.y + tap / 3 - 1, sx = px.x + tap % 3 - 1;
                    if (sy >= 0 && sy < H && sx >= 0 && sx < W) b = load_cat8(x1, C1, x2, C2, px.n, sy, sx, H, W, ci);
                }
            }
            ra[i] = a;
            rb[i] = b;
        }
    };
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
    const int nk = (pend - pbeg + BK - 1) / BK;
    if (nk > 0) load(pbeg);
    for (int kt = 0; kt < nk; ++kt) {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int v = tid + i * NT;
            *(uint4*)(At + (v >> 3) * TP + (v & 7) * 8) = ra[i];
            *(uint4*)(Bt + (v >> 3) * TP + (v & 7) * 8) = rb[i];
        }
        __syncthreads();
        if (kt + 1 < nk) load(pbeg + (kt + 1) * BK);
        mma_chunk<true, true>(At, Bt, acc, wm, wn, lane);
        __syncthreads();
    }
    const int g = lane >> 2, c4 = lane & 3;
    float* out = ws + (size_t)blockIdx.z * Cout * N9;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int co = m0 + wm * 32 + mt * 16 + g + 8 * h2;
                const int n = n0 + wn * 32 + nt * 8 + 2 * c4;
                if (co < Cout && n < N9)
                    *(float2*)(out + (size_t)co * N9 + n) = make_float2(acc[mt][nt][2 * h2], acc[mt][nt][2 * h2 + 1]);
            }
}

__global__ void k_sum_splits(const float* __restrict__ ws, int nz, long long size, float* __restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < size; i += (long long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int z = 0; z < nz; ++z) s += ws[(size_t)z * size + i];
        out[i] = s;
    }
}

// bias gradient, stage 1: per block of kBiasRows pixels, per channel.  Thread
// (lane of pixels pl, channel group cg) adds 8 channels (one 16-byte load of dy,
// and of y for the ReLU derivative) of pixels pl, pl + lanes, ...; the pixel
// lanes' sums are then added in a fixed order in shared memory.
constexpr int kBiasRows = 512;
constexpr int kBiasThreads = 256;
template <int RELU>
__global__ void __launch_bounds__(kBiasThreads)
k_bias_partial(const bf16* __restrict__ dy, const bf16* __restrict__ yv, int P, int Cout, float* __restrict__ part) {
    __shared__ float red[kBiasThreads * 8];
    const int groups = Cout / 8;
    const int G = groups < kBiasThreads ? groups : kBiasThreads;
    const int lanes = kBiasThreads / G;
    const int cg0 = threadIdx.x % G, pl = threadIdx.x / G;
    const int p0 = blockIdx.x * kBiasRows, p1 = min(P, p0 + kBiasRows);
    for (int cb = 0; cb < groups; cb += G) {
        const int cg = cb + cg0;
        float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (pl < lanes && cg < groups) {
            for (int p = p0 + pl; p < p1; p += lanes) {
                const size_t q = (size_t)p * Cout + cg * 8;
                uint4 d = *(const uint4*)(dy + q);
                if (RELU) d = relu_mask8(d, *(const uint4*)(yv + q));
                const __nv_bfloat162* h = (const __nv_bfloat162*)&d;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float2 f = __bfloat1622float2(h[k]);
                    s[2 * k] += f.x;
                    s[2 * k + 1] += f.y;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) red[threadIdx.x * 8 + k] = s[k];
        __syncthreads();
        for (int e = threadIdx.x; e < G * 8; e += kBiasThreads) {
            const int g = e / 8, k = e % 8;
            if (cb + g < groups) {
                float t = 0.f;
                for (int l = 0; l < lanes; ++l) t += red[(l * G + g) * 8 + k];
                part[(size_t)blockIdx.x * Cout + (cb + g) * 8 + k] = t;
            }
        }
        __syncthreads();
    }
}

// bias gradient, stage 2: one block per channel adds the blocks' partial sums
// (strided per thread, then a fixed tree)
__global__ void __launch_bounds__(256) k_bias_reduce(const float* __restrict__ part, int nblk, int Cout,
                                                     float* __restrict__ db) {
    __shared__ float red[256];
    const int co = blockIdx.x;
    float s = 0.f;
    for (int b = threadIdx.x; b < nblk; b += 256) s += part[(size_t)b * Cout + co];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[co] = red[0];
}

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------
__global__ void k_prep_weights(const float* __restrict__ w, bf16* __restrict__ wb, bf16* __restrict__ wt, int Cout,
                               int Cin) {
    const int K = 9 * Cin;
    const long long total = (long long)Cout * K;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int co = (int)(i / K), k = (int)(i - (long long)co * K);
        const bf16 v = __float2bfloat16_rn(w[i]);
        if (wb) wb[i] = v;
        if (wt) wt[(size_t)k * Cout + co] = v;  // k = tap * Cin + ci
    }
}

__device__ __forceinline__ void unpack8(uint4 u, float (&f)[8]) {
    const __nv_bfloat162* h = (const __nv_bfloat162*)&u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    uint4 u;
    __nv_bfloat162* h = (__nv_bfloat162*)&u;
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    return u;
}

// y (n, h/2, w/2, c) = mean of the 2x2 block of x (n, h, w, c); one thread per 8 channels
__global__ void k_pool2_fwd(const bf16* __restrict__ x, bf16* __restrict__ y, int NB, int H, int W, int C) {
    const int h2 = H / 2, w2 = W / 2, c8 = C / 8;
    const long long total = (long long)NB * h2 * w2 * c8;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int cv = (int)(t % c8);
        long long r = t / c8;
        const int j = (int)(r % w2);
        r /= w2;
        const int i = (int)(r % h2);
        const int n = (int)(r / h2);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0}, f[8];
#pragma unroll
        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
            for (int dx = 0; dx < 2; ++dx) {
                unpack8(*(const uint4*)(x + (((size_t)n * H + 2 * i + dy) * W + 2 * j + dx) * C + cv * 8), f);
#pragma unroll
                for (int q = 0; q < 8; ++q) s[q] += f[q];
            }
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] *= 0.25f;
        *(uint4*)(y + (((size_t)n * h2 + i) * w2 + j) * C + cv * 8) = pack8(s);
    }
}

// dx (n, h, w, c) = dy (n, h/2, w/2, c) / 4
__global__ void k_pool2_bwd(const bf16* __restrict__ dy, bf16* __restrict__ dx, int NB, int H, int W, int C) {
    const int c8 = C / 8;
    const long long total = (long long)NB * H * W * c8;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int cv = (int)(t % c8);
        long long r = t / c8;
        const int x = (int)(r % W);
        r /= W;
        const int yy = (int)(r % H);
        const int n = (int)(r / H);
        float f[8];
        unpack8(*(const uint4*)(dy + (((size_t)n * (H / 2) + yy / 2) * (W / 2) + x / 2) * C + cv * 8), f);
#pragma unroll
        for (int q = 0; q < 8; ++q) f[q] *= 0.25f;
        *(uint4*)(dx + (((size_t)n * H + yy) * W + x) * C + cv * 8) = pack8(f);
    }
}

// y (n, h, w, c) = x (n, h/2, w/2, c)
__global__ void k_up2_fwd(const bf16* __restrict__ x, bf16* __restrict__ y, int NB, int H, int W, int C) {
    const int c8 = C / 8;
    const long long total = (long long)NB * H * W * c8;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int cv = (int)(t % c8);
        long long r = t / c8;
        const int xx = (int)(r % W);
        r /= W;
        const int yy = (int)(r % H);
        const int n = (int)(r / H);
        *(uint4*)(y + (((size_t)n * H + yy) * W + xx) * C + cv * 8) =
            *(const uint4*)(x + (((size_t)n * (H / 2) + yy / 2) * (W / 2) + xx / 2) * C + cv * 8);
    }
}

// dx (n, h/2, w/2, c) = sum of the 2x2 block of dy (n, h, w, c)
__global__ void k_up2_bwd(const bf16* __restrict__ dy, bf16* __restrict__ dx, int NB, int H, int W, int C) {
    const int h2 = H / 2, w2 = W / 2, c8 = C / 8;
    const long long total = (long long)NB * h2 * w2 * c8;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int cv = (int)(t % c8);
        long long r = t / c8;
        const int j = (int)(r % w2);
        r /= w2;
        const int i = (int)(r % h2);
        const int n = (int)(r / h2);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0}, f[8];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                unpack8(*(const uint4*)(dy + (((size_t)n * H + 2 * i + a) * W + 2 * j + b) * C + cv * 8), f);
#pragma unroll
                for (int q = 0; q < 8; ++q) s[q] += f[q];
            }
        *(uint4*)(dx + (((size_t)n * h2 + i) * w2 + j) * C + cv * 8) = pack8(s);
    }
}

__global__ void k_add(const bf16* __restrict__ a, const bf16* __restrict__ b, bf16* __restrict__ out, long long n8) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n8; t += (long long)gridDim.x * blockDim.x) {
        float fa[8], fb[8];
        unpack8(((const uint4*)a)[t], fa);
        unpack8(((const uint4*)b)[t], fb);
#pragma unroll
        for (int q = 0; q < 8; ++q) fa[q] += fb[q];
        ((uint4*)out)[t] = pack8(fa);
    }
}

constexpr int kLossBlocks = 512;
__global__ void k_mse(const bf16* __restrict__ pred, int cp, const float* __restrict__ tgt, int ct,
                      const float* __restrict__ cw, bf16* __restrict__ dpred, float* __restrict__ part, long long npix) {
    __shared__ float sm[256];
    float s = 0.f;
    const float inv = 1.f / (float)npix;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        for (int c = 0; c < cp; ++c) {
            float d = 0.f;
            if (c < ct) {
                const float e = __bfloat162float(pred[p * cp + c]) - tgt[p * ct + c];
                s += cw[c] * e * e;
                d = 2.f * cw[c] * e * inv;
            }
            dpred[p * cp + c] = __float2bfloat16_rn(d);
        }
    }
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_mse_finish(const float* __restrict__ part, int nb, long long npix, float* __restrict__ loss) {
    __shared__ float sm[256];
    float s = 0.f;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[0] = sm[0] / (float)npix;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long n, float lr, float b1, float b2, float eps, float wd, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / c1, vh = vi / c2;
        w[i] -= lr * (mh / (sqrtf(vh) + eps) + wd * w[i]);
    }
}

__global__ void k_f2b(const float* __restrict__ x, bf16* __restrict__ y, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}
__global__ void k_b2f(const bf16* __restrict__ x, float* __restrict__ y, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __bfloat162float(x[i]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static inline int ret(cudaError_t e) { return e == cudaSuccess ? GLGPU_OK : GLGPU_E_CUDA; }
static inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
static inline int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    return (int)std::max(1LL, std::min(b, 152LL * 32));
}
static inline bool conv_shape_ok(int c1, int c2, int n, int h, int w, int cout) {
    return n > 0 && h > 0 && w > 0 && c1 > 0 && c1 % 8 == 0 && c2 >= 0 && c2 % 8 == 0 && cout > 0 && cout % 8 == 0 &&
           (long long)n * h * w < (1LL << 31);
}

// split-K plan of the weight gradient
struct WPlan {
    int nz, chunk, tiles, nbias;
    long long ws_floats, bias_floats;
};
static WPlan wplan(int n, int h, int w, int cin, int cout) {
    WPlan q;
    const long long P = (long long)n * h * w;
    q.tiles = ((cout + BM - 1) / BM) * ((9 * cin + BN - 1) / BN);
    long long nz = (4 * 152 + q.tiles - 1) / q.tiles;
    const long long kmax = (P + BK - 1) / BK;
    nz = std::max(1LL, std::min(nz, kmax));
    long long chunk = ((P + nz - 1) / nz + BK - 1) / BK * BK;
    q.nz = (int)((P + chunk - 1) / chunk);
    q.chunk = (int)chunk;
    q.ws_floats = (long long)q.nz * cout * 9 * cin;
    q.nbias = (int)((P + kBiasRows - 1) / kBiasRows);
    q.bias_floats = (long long)q.nbias * cout;
    return q;
}

}  // namespace glnn

using namespace glnn;

// nn_tc.cu: the weight gradient on tcgen05 with TMA operands (its split plan, and
// the launch: 1 when enqueued, 0 when the shape or the TMA switch rule it out)
void glnn_tc_wgrad_plan(int n, int h, int w, int cin, int cout, int* nz, int* chunk);
int glnn_tc_wgrad(const void* dy, const void* y, int relu, const void* x1, int c1, const void* x2, int c2, float* ws,
                  void* dy_masked, int n, int h, int w, int cout, int* err, cudaStream_t s);

// work layout: [split partial sums (the larger of the two plans)][bias partials]
// [dy * relu'(y) in bf16, for the tcgen05 path], each part 256-byte aligned
struct WLayout {
    long long ws, bias_off, dym_off, total;
};
static WLayout wlayout(int n, int h, int w, int cin, int cout) {
    const WPlan q = wplan(n, h, w, cin, cout);
    int nz_tc = 0, chunk_tc = 0;
    glnn_tc_wgrad_plan(n, h, w, cin, cout, &nz_tc, &chunk_tc);
    auto up = [](long long v) { return (v + 63) / 64 * 64; };
    WLayout L;
    L.ws = up(std::max(q.ws_floats, (long long)nz_tc * cout * 9 * cin));
    L.bias_off = L.ws;
    L.dym_off = L.bias_off + up(q.bias_floats);
    L.total = L.dym_off + up(((long long)n * h * w * cout + 1) / 2);
    return L;
}

extern "C" {

int64_t glnn_conv3x3_bwd_weight_work(int32_t n, int32_t h, int32_t w, int32_t cin, int32_t cout) {
    if (n <= 0 || h <= 0 || w <= 0 || cin <= 0 || cout <= 0) return 0;
    return wlayout(n, h, w, cin, cout).total;
}

int glnn_conv3x3_bwd_weight(const void* dy, const void* y, int32_t relu, const void* x1, int32_t c1, const void* x2,
                            int32_t c2, float* dw, float* db, float* work, int64_t work_floats, int32_t n, int32_t h,
                            int32_t w, int32_t cout, int32_t* err, void* stream) {
    if (!dy || !x1 || !dw || !db || !work || !err || (relu && !y) || (c2 > 0 && !x2) ||
        !conv_shape_ok(c1, c2, n, h, w, cout))
        return GLGPU_E_ARG;
    if (!aligned16(dy) || (y && !aligned16(y)) || !aligned16(x1) || (x2 && !aligned16(x2)) || !aligned16(work))
        return GLGPU_E_ARG;
    const int cin = c1 + c2;
    const WPlan q = wplan(n, h, w, cin, cout);
    const WLayout L = wlayout(n, h, w, cin, cout);
    if (work_floats < L.total) return GLGPU_E_ARG;
    const long long P = (long long)n * h * w;
    cudaStream_t s = (cudaStream_t)stream;
    float* bias_part = work + L.bias_off;
    int nz = q.nz;
    if (glnn_tc_wgrad(dy, y, relu, x1, c1, x2, c2, work, work + L.dym_off, n, h, w, cout, err, s)) {
        int chunk_tc = 0;
        glnn_tc_wgrad_plan(n, h, w, cin, cout, &nz, &chunk_tc);
    } else {
        dim3 grid((unsigned)((cout + BM - 1) / BM), (unsigned)((9 * cin + BN - 1) / BN), (unsigned)q.nz);
        if (relu)
            k_conv_bwd_weight<1><<<grid, NT, 0, s>>>((const bf16*)dy, (const bf16*)y, (const bf16*)x1, c1, (const bf16*)x2, c2, work, n, h, w, cout, q.chunk);
        else
            k_conv_bwd_weight<0><<<grid, NT, 0, s>>>((const bf16*)dy, (const bf16*)y, (const bf16*)x1, c1, (const bf16*)x2, c2, work, n, h, w, cout, q.chunk);
    }
    if (relu)
        k_bias_partial<1><<<q.nbias, kBiasThreads, 0, s>>>((const bf16*)dy, (const bf16*)y, (int)P, cout, bias_part);
    else
        k_bias_partial<0><<<q.nbias, kBiasThreads, 0, s>>>((const bf16*)dy, (const bf16*)y, (int)P, cout, bias_part);
    const long long size = (long long)cout * 9 * cin;
    k_sum_splits<<<grid_for(size, 256), 256, 0, s>>>(work, nz, size, dw);
    k_bias_reduce<<<cout, 256, 0, s>>>(bias_part, q.nbias, cout, db);
    return ret(cudaGetLastError());
}

int glnn_prep_weights(const float* w, void* wb, void* wt, int32_t cout, int32_t cin, void* stream) {
    if (!w || cout <= 0 || cin <= 0) return GLGPU_E_ARG;
    const long long total = (long long)cout * 9 * cin;
    k_prep_weights<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>(w, (bf16*)wb, (bf16*)wt, cout, cin);
    return ret(cudaGetLastError());
}

static bool pool_ok(const void* a, const void* b, int n, int h, int w, int c) {
    return a && b && n > 0 && h > 1 && w > 1 && h % 2 == 0 && w % 2 == 0 && c > 0 && c % 8 == 0 && aligned16(a) &&
           aligned16(b);
}

int glnn_pool2_fwd(const void* x, void* y, int32_t n, int32_t h, int32_t w, int32_t c, void* stream) {
    if (!pool_ok(x, y, n, h, w, c)) return GLGPU_E_ARG;
    const long long total = (long long)n * (h / 2) * (w / 2) * (c / 8);
    k_pool2_fwd<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)y, n, h, w, c);
    return ret(cudaGetLastError());
}

int glnn_pool2_bwd(const void* dy, void* dx, int32_t n, int32_t h, int32_t w, int32_t c, void* stream) {
    if (!pool_ok(dy, dx, n, h, w, c)) return GLGPU_E_ARG;
    const long long total = (long long)n * h * w * (c / 8);
    k_pool2_bwd<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>((const bf16*)dy, (bf16*)dx, n, h, w, c);
    return ret(cudaGetLastError());
}

int glnn_up2_fwd(const void* x, void* y, int32_t n, int32_t h, int32_t w, int32_t c, void* stream) {
    if (!pool_ok(x, y, n, h, w, c)) return GLGPU_E_ARG;
    const long long total = (long long)n * h * w * (c / 8);
    k_up2_fwd<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)y, n, h, w, c);
    return ret(cudaGetLastError());
}

int glnn_up2_bwd(const void* dy, void* dx, int32_t n, int32_t h, int32_t w, int32_t c, void* stream) {
    if (!pool_ok(dy, dx, n, h, w, c)) return GLGPU_E_ARG;
    const long long total = (long long)n * (h / 2) * (w / 2) * (c / 8);
    k_up2_bwd<<<grid_for(total, 256), 256, 0, (cudaStream_t)stream>>>((const bf16*)dy, (bf16*)dx, n, h, w, c);
    return ret(cudaGetLastError());
}

int glnn_add(const void* a, const void* b, void* out, int64_t count, void* stream) {
    if (!a || !b || !out || count < 0 || count % 8 || !aligned16(a) || !aligned16(b) || !aligned16(out)) return GLGPU_E_ARG;
    k_add<<<grid_for(count / 8, 256), 256, 0, (cudaStream_t)stream>>>((const bf16*)a, (const bf16*)b, (bf16*)out, count / 8);
    return ret(cudaGetLastError());
}

int glnn_mse(const void* pred, int32_t cp, const float* target, int32_t ct, const float* cw, void* dpred, float* loss,
             float* work, int64_t npix, void* stream) {
    if (!pred || !target || !cw || !dpred || !loss || !work || cp <= 0 || ct <= 0 || ct > cp || npix <= 0) return GLGPU_E_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    k_mse<<<kLossBlocks, 256, 0, s>>>((const bf16*)pred, cp, target, ct, cw, (bf16*)dpred, work, npix);
    k_mse_finish<<<1, 256, 0, s>>>(work, kLossBlocks, npix, loss);
    return ret(cudaGetLastError());
}

int glnn_adam(float* w, const float* g, float* m, float* v, int64_t count, float lr, float beta1, float beta2,
              float eps, float weight_decay, int32_t step, void* stream) {
    if (!w || !g || !m || !v || count < 0 || step < 1) return GLGPU_E_ARG;
    const float c1 = 1.f - (float)std::pow((double)beta1, (double)step);
    const float c2 = 1.f - (float)std::pow((double)beta2, (double)step);
    k_adam<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, count, lr, beta1, beta2, eps, weight_decay, c1, c2);
    return ret(cudaGetLastError());
}

int glnn_f32_to_bf16(const float* x, void* y, int64_t count, void* stream) {
    if (!x || !y || count < 0) return GLGPU_E_ARG;
    k_f2b<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>(x, (bf16*)y, count);
    return ret(cudaGetLastError());
}

int glnn_bf16_to_f32(const void* x, float* y, int64_t count, void* stream) {
    if (!x || !y || count < 0) return GLGPU_E_ARG;
    k_b2f<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>((const bf16*)x, y, count);
    return ret(cudaGetLastError());
}

}  // extern "C"
