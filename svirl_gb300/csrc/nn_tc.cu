// Forward 3x3 convolution of the learned warm start on the 5th-generation tensor
// cores: tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in tensor
// memory), one 128 x 64 output tile per CTA.  Per K chunk of 64 the four warps
// gather the implicit-GEMM operands (pixels x [tap, cin] of the input, cout x
// [tap, cin] of the weights) into shared memory in the K-major core-matrix
// layout (8 rows x 16 bytes per core matrix, no swizzle), one thread issues four
// 128x64x16 MMAs and commits them to an mbarrier, and the CTA waits on it before
// the next chunk overwrites the operands.  The epilogue reads the accumulator
// with tcgen05.ld (each warp its 32 TMEM lanes = 32 output pixels), adds the
// bias, applies the ReLU and stores bfloat16.  Every wait is bounded; on a
// timeout the kernel records an error, skips its stores and still frees its
// tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/glgpu.h"
#include "../../include/glgpu_nn.h"

namespace glnn_tc {

typedef __nv_bfloat16 bf16;

constexpr int TM = 128, TN = 64, TK = 64, NTH = 128;
constexpr int A_BYTES = TM * TK * 2;        // 16 KB
constexpr int B_BYTES = TN * TK * 2;        // 8 KB
constexpr int SMEM_BYTES = A_BYTES + B_BYTES + 16;
constexpr uint32_t kTmemCols = 64;          // FP32 accumulator: TN columns
constexpr uint32_t kSpinLimit = 1u << 20;   // mbarrier polls before giving up
// instruction descriptor (kind::f16): D f32 (bits 4-5 = 1), A bf16 (7-9 = 1),
// B bf16 (10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at 17-22, M >> 4 at 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (row, k) of a K-major tile with `kb` core matrices along K:
// core matrix (row / 8, k / 8) at ((row / 8) * kb + k / 8) * 128 B, rows of 16 B inside.
__device__ __forceinline__ int core_off(int row, int k, int kb) {
    return ((((row >> 3) * kb) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
}

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), leading-dimension
// byte offset >> 4 (16-29: next core matrix along K), stride byte offset >> 4
// (32-45: next 8-row group), version 1 (46-47), no swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t start, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((start >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    return d;
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t phase) {
    for (uint32_t it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ uint4 load_cat8(const bf16* x1, int C1, const bf16* x2, int C2, int n, int sy, int sx,
                                           int H, int W, int ci) {
    const size_t q = ((size_t)n * H + sy) * W + sx;
    return ci < C1 ? *(const uint4*)(x1 + q * C1 + ci) : *(const uint4*)(x2 + q * C2 + (ci - C1));
}

template <int RELU>
__global__ void __launch_bounds__(NTH)
k_conv_fwd_tc(const bf16* __restrict__ x1, int C1, const bf16* __restrict__ x2, int C2, const bf16* __restrict__ Wb,
              const float* __restrict__ bias, bf16* __restrict__ y, int NB, int H, int W, int Cout, int* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* As = smem;
    unsigned char* Bs = smem + A_BYTES;
    uint64_t* bar = (uint64_t*)(smem + A_BYTES + B_BYTES);
    uint32_t* tslot = (uint32_t*)(smem + A_BYTES + B_BYTES + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Cin = C1 + C2, K = 9 * Cin, P = NB * H * W;
    const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;

    // the 8 A rows (pixels) this thread gathers: row = (tid + 128 i) >> 3 = tid / 8 + 16 i
    int pn[8], py[8], px[8];
    bool pok[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int p = m0 + ((tid + i * NTH) >> 3);
        pok[i] = p < P;
        const int pp = pok[i] ? p : 0;
        px[i] = pp % W;
        py[i] = (pp / W) % H;
        pn[i] = pp / (W * H);
    }
    const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
    const int nk = (K + TK - 1) / TK;
    uint32_t phase = 0;
    bool ok = true;
    for (int kt = 0; kt < nk; ++kt) {
        const int kc = kt * TK;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int v = tid + i * NTH, row = v >> 3, kv = v & 7, k = kc + kv * 8;
            uint4 a = z4;
            if (pok[i] && k < K) {
                const int tap = k / Cin, ci = k - tap * Cin;
                const int sy = py[i] + tap / 3 - 1, sx = px[i] + tap % 3 - 1;
                if (sy >= 0 && sy < H && sx >= 0 && sx < W) a = load_cat8(x1, C1, x2, C2, pn[i], sy, sx, H, W, ci);
            }
            *(uint4*)(As + core_off(row, kv * 8, TK / 8)) = a;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int v = tid + i * NTH, row = v >> 3, kv = v & 7, k = kc + kv * 8;
            const int co = n0 + row;
            const uint4 b = (co < Cout && k < K) ? *(const uint4*)(Wb + (size_t)co * K + k) : z4;
            *(uint4*)(Bs + core_off(row, kv * 8, TK / 8)) = b;
        }
        // generic-proxy stores -> visible to the tensor core's (async-proxy) reads
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int j = 0; j < TK / 16; ++j) {
                const uint64_t ad = smem_desc(saddr(As) + j * 256, 128, 1024);
                const uint64_t bd = smem_desc(saddr(Bs) + j * 256, 128, 1024);
                mma_f16(tmem, ad, bd, kIdesc, (kt > 0 || j > 0) ? 1u : 0u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             saddr(bar))
                         : "memory");
        }
        // the MMAs read As/Bs: wait for them before the next chunk overwrites
        const bool got = wait_parity(saddr(bar), phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (__syncthreads_or(got ? 0 : 1)) {
            ok = false;
            break;
        }
    }
    if (ok) {
        const int p = m0 + warp * 32 + lane;  // TMEM lane = output row
#pragma unroll
        for (int c = 0; c < TN; c += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (p < P) {
#pragma unroll
                for (int q = 0; q < 16; q += 2) {
                    const int col = n0 + c + q;
                    if (col < Cout) {
                        float v0 = __uint_as_float(r[q]) + bias[col], v1 = __uint_as_float(r[q + 1]) + bias[col + 1];
                        if (RELU) {
                            v0 = fmaxf(v0, 0.f);
                            v1 = fmaxf(v1, 0.f);
                        }
                        *(__nv_bfloat162*)(y + (size_t)p * Cout + col) = __floats2bfloat162_rn(v0, v1);
                    }
                }
            }
        }
    } else {
        // a commit that never arrived: wait once more (bounded) before the memory goes
        wait_parity(saddr(bar), phase ^ 1u);
        if (tid == 0) atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace glnn_tc

using namespace glnn_tc;

extern "C" {

int glnn_conv3x3_fwd_tc(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* wb, const float* bias,
                        void* y, int32_t n, int32_t h, int32_t w, int32_t cout, int32_t relu, int32_t* err,
                        void* stream) {
    if (!x1 || !wb || !bias || !y || !err || (c2 > 0 && !x2)) return GLGPU_E_ARG;
    if (n <= 0 || h <= 0 || w <= 0 || c1 <= 0 || c1 % 8 || c2 < 0 || c2 % 8 || cout <= 0 || cout % 8) return GLGPU_E_ARG;
    if ((long long)n * h * w >= (1LL << 31)) return GLGPU_E_ARG;
    if (((uintptr_t)x1 | (uintptr_t)x2 | (uintptr_t)wb | (uintptr_t)y) & 15u) return GLGPU_E_ARG;
    const long long P = (long long)n * h * w;
    dim3 grid((unsigned)((P + TM - 1) / TM), (unsigned)((cout + TN - 1) / TN));
    cudaStream_t s = (cudaStream_t)stream;
    if (relu)
        k_conv_fwd_tc<1><<<grid, NTH, SMEM_BYTES, s>>>((const bf16*)x1, c1, (const bf16*)x2, c2, (const bf16*)wb, bias,
                                                      (bf16*)y, n, h, w, cout, err);
    else
        k_conv_fwd_tc<0><<<grid, NTH, SMEM_BYTES, s>>>((const bf16*)x1, c1, (const bf16*)x2, c2, (const bf16*)wb, bias,
                                                      (bf16*)y, n, h, w, cout, err);
    return cudaGetLastError() == cudaSuccess ? GLGPU_OK : GLGPU_E_CUDA;
}

}  // extern "C"
