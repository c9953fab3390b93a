// 3x3 convolutions of the learned warm start on the 5th-generation tensor cores:
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator in tensor memory), one
// 128 x 64 output tile per CTA, for the forward pass (M = pixels, N = cout,
// K = [tap, cin] of the input shifted by the tap) and the data gradient
// (M = pixels, N = cin, K = [tap, cout] of dy shifted back, with the layer's
// ReLU derivative applied while gathering).  Per K chunk of 64 the four warps
// gather the implicit-GEMM operands into shared memory in the K-major core-matrix
// layout (8 rows x 16 bytes per core matrix, no swizzle), one thread issues four
// 128x64x16 MMAs and commits them to the stage's mbarrier, and the loads of the
// next chunk go out while they run; a stage is refilled only after the MMAs that
// read it have signalled completion.  One stage (24 KB) keeps about nine CTAs per
// SM; two stages measured slower (fewer CTAs per SM).  The epilogue reads the accumulator
// with tcgen05.ld (each warp its 32 TMEM lanes = 32 output pixels), adds the
// bias, applies the ReLU and stores bfloat16.  Every wait is bounded; on a
// timeout the kernel records an error, skips its stores and still frees its
// tensor memory.  The weight gradient (K = pixels) is in nn.cu.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "../../include/glgpu.h"
#include "../../include/glgpu_nn.h"

namespace glnn_tc {

typedef __nv_bfloat16 bf16;

constexpr int TM = 128, TN = 64, TK = 64, NTH = 128;
constexpr int A_BYTES = TM * TK * 2;        // 16 KB
constexpr int B_BYTES = TN * TK * 2;        // 8 KB
#ifndef GLNN_TC_STAGES
#define GLNN_TC_STAGES 1
#endif
constexpr int kStages = GLNN_TC_STAGES;       // operand stages in shared memory (1 or 2)
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int SMEM_BYTES = kStages * STAGE_BYTES + 32;  // stages, a barrier per stage, the TMEM address
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

// dy * (y > 0) on packed bf16 values (y > 0: sign clear and not zero)
__device__ __forceinline__ uint32_t relu_mask2(uint32_t d, uint32_t y) {
    const uint32_t lo = ((y & 0xffffu) - 1u) < 0x7fffu ? 0x0000ffffu : 0u;
    const uint32_t hi = ((y >> 16) - 1u) < 0x7fffu ? 0xffff0000u : 0u;
    return d & (lo | hi);
}

// MODE 0 (forward): A = [x1 | x2] shifted by +tap, B = Wb[n][k], out = y (+ bias, ReLU).
// MODE 1 (data gradient): A = dy * relu'(mask) shifted by -tap (a1 = dy, Ca1 = cout),
// B = Wt[tap][n][c], out = [o1 | o2] (the input's two channel groups).
template <int MODE, int RELU>
__global__ void __launch_bounds__(NTH)
k_conv_tc(const bf16* __restrict__ a1, int Ca1, const bf16* __restrict__ a2, int Ca2, const bf16* __restrict__ mask,
          const bf16* __restrict__ Bsrc, const float* __restrict__ bias, bf16* __restrict__ o1, int Co1,
          bf16* __restrict__ o2, int Co2, int NB, int H, int W, int* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* bar = (uint64_t*)(smem + kStages * STAGE_BYTES);  // bar[s]: MMAs of stage s done
    uint32_t* tslot = (uint32_t*)(smem + kStages * STAGE_BYTES + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Ca = Ca1 + Ca2, K = 9 * Ca, Nout = Co1 + Co2, P = NB * H * W;
    const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < kStages; ++q)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(bar + q)) : "memory");
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
    // operands of the next chunk are loaded into registers while the tensor core
    // works on the current one; two shared-memory stages, each reused only after
    // the MMAs that read it (two chunks earlier) have completed
    uint4 ra[8], rb[4];
    auto gather = [&](int kc) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int kv = (tid + i * NTH) & 7, k = kc + kv * 8;
            uint4 a = z4;
            if (pok[i] && k < K) {
                const int tap = k / Ca, c = k - tap * Ca;
                const int dy = MODE == 0 ? tap / 3 - 1 : 1 - tap / 3, dx = MODE == 0 ? tap % 3 - 1 : 1 - tap % 3;
                const int sy = py[i] + dy, sx = px[i] + dx;
                if (sy >= 0 && sy < H && sx >= 0 && sx < W) {
                    a = load_cat8(a1, Ca1, a2, Ca2, pn[i], sy, sx, H, W, c);
                    if (MODE == 1 && RELU) {
                        const uint4 m = *(const uint4*)(mask + (((size_t)pn[i] * H + sy) * W + sx) * Ca1 + c);
                        a = make_uint4(relu_mask2(a.x, m.x), relu_mask2(a.y, m.y), relu_mask2(a.z, m.z),
                                       relu_mask2(a.w, m.w));
                    }
                }
            }
            ra[i] = a;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int v = tid + i * NTH, row = v >> 3, kv = v & 7, k = kc + kv * 8;
            const int nn = n0 + row;
            uint4 b = z4;
            if (nn < Nout && k < K) {
                if (MODE == 0) {
                    b = *(const uint4*)(Bsrc + (size_t)nn * K + k);
                } else {
                    const int tap = k / Ca, c = k - tap * Ca;
                    b = *(const uint4*)(Bsrc + ((size_t)tap * Nout + nn) * Ca + c);
                }
            }
            rb[i] = b;
        }
    };
    uint32_t phase[2] = {0u, 0u};
    bool ok = true;
    gather(0);
    for (int kt = 0; kt < nk; ++kt) {
        const int st = kt % kStages;
        unsigned char* As = smem + st * STAGE_BYTES;
        unsigned char* Bs = As + A_BYTES;
        if (kt >= kStages) {  // the MMAs of chunk kt - kStages read this stage
            const bool got = wait_parity(saddr(bar + st), phase[st]);
            phase[st] ^= 1u;
            if (__syncthreads_or(got ? 0 : 1)) {
                ok = false;
                break;
            }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int v = tid + i * NTH;
            *(uint4*)(As + core_off(v >> 3, (v & 7) * 8, TK / 8)) = ra[i];
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int v = tid + i * NTH;
            *(uint4*)(Bs + core_off(v >> 3, (v & 7) * 8, TK / 8)) = rb[i];
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
                             saddr(bar + st))
                         : "memory");
        }
        if (kt + 1 < nk) gather((kt + 1) * TK);
    }
    // each stage's most recent commit (the last kStages chunks)
    for (int q = nk >= kStages ? nk - kStages : 0; q < nk; ++q) {
        const int st = q % kStages;
        const bool got = wait_parity(saddr(bar + st), phase[st]);
        phase[st] ^= 1u;
        if (!got) ok = false;
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (__syncthreads_or(ok ? 0 : 1)) ok = false;
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
                    if (col < Nout) {
                        float v0 = __uint_as_float(r[q]), v1 = __uint_as_float(r[q + 1]);
                        if (MODE == 0) {
                            v0 += bias[col];
                            v1 += bias[col + 1];
                            if (RELU) {
                                v0 = fmaxf(v0, 0.f);
                                v1 = fmaxf(v1, 0.f);
                            }
                        }
                        const __nv_bfloat162 v = __floats2bfloat162_rn(v0, v1);
                        if (col < Co1) *(__nv_bfloat162*)(o1 + (size_t)p * Co1 + col) = v;
                        else *(__nv_bfloat162*)(o2 + (size_t)p * Co2 + (col - Co1)) = v;
                    }
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// ---------------------------------------------------------------------------
// Forward 3x3 convolution with the operands loaded by TMA (cp.async.bulk.tensor).
// For layers whose input and output channel counts are multiples of 64 and whose
// 128-pixel tiles are whole image rows (W a multiple of 128) or whole groups of
// rows (128 a multiple of W), the A operand of tap (dy, dx) and channel chunk
// c0..c0+63 is one box of the input viewed as the 4-D tensor [n][h][w][c]: the
// tile's rows shifted by (dy, dx); the copy engine writes zeros where the box
// leaves the image, which is the "same" padding.  B (the weights [cout][9 cin])
// is a 64 x 64 box of a 2-D tensor.  Both land in shared memory in the 128-byte
// swizzled K-major layout the MMA descriptors name (layout type 2).  Thread 0
// issues the copies into a 4-stage ring (full barrier: the stage's bytes),
// thread 32 issues four 128x64x16 tcgen05 MMAs per chunk and commits them to the
// stage's empty barrier; all four warps then read the accumulator (TMEM lane =
// output pixel) for the bias + ReLU epilogue.  Waits are bounded.
// ---------------------------------------------------------------------------
#ifndef GLNN_TMA_STAGES
#define GLNN_TMA_STAGES 2
#endif
constexpr int TMA_STAGES = GLNN_TMA_STAGES;  // operand stages of the TMA forward / data gradient
// stages, 1024-byte alignment slack, then the barriers (full and empty per stage, done)
// and the TMEM address slot
constexpr int TMA_SMEM = TMA_STAGES * STAGE_BYTES + 1024 + (2 * TMA_STAGES + 2) * 8;
constexpr uint32_t kStageTx = (uint32_t)STAGE_BYTES;
static_assert(TMA_STAGES >= 1 && TMA_SMEM <= 227 * 1024, "TMA conv stages exceed shared memory");

// SM100 shared-memory matrix descriptor, K-major with the 128-byte swizzle:
// start >> 4 (bits 0-13), leading offset 16 B (unused for this layout), stride
// offset 1024 B between 8-row groups (32-45), version 1 (46-47), layout type
// 2 = 128-byte swizzle (61-63).  A K step of 16 elements advances the start by 32 B.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t start) {
    uint64_t d = (uint64_t)((start >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// MODE 0 (forward): A = [x1 | x2] (C1 + C2 channels) shifted by +tap, B = Wb as the
// 2-D tensor [cout][9 cin] (box: 64 rows of 64 k), out = y (Co1 = cout channels,
// + bias, ReLU).  MODE 1 (data gradient): A = dy' (C1 = cout channels, C2 = 0: dy
// with the ReLU derivative already applied) shifted by -tap, B = Wt as the 3-D
// tensor [9][cin][cout] (box: 64 cin rows of 64 cout, one tap), out = [o1 | o2]
// (Co1 + Co2 = cin channels), no bias.
template <int MODE, int RELU>
__global__ void __launch_bounds__(NTH)
k_conv_fwd_tma(const __grid_constant__ CUtensorMap ta1, const __grid_constant__ CUtensorMap ta2,
               const __grid_constant__ CUtensorMap tb, const float* __restrict__ bias, bf16* __restrict__ y, int Cout,
               bf16* __restrict__ o2, int Co2, int C1, int C2, int H, int W, int* err) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + TMA_STAGES * STAGE_BYTES);
    uint64_t* empty = full + TMA_STAGES;
    uint64_t* done = empty + TMA_STAGES;
    uint32_t* tslot = (uint32_t*)(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
    const int img = m0 / (H * W), rem = m0 - img * H * W, y0 = rem / W, x0 = rem - y0 * W;
    const int nck = (C1 + C2) / TK, nk = 9 * nck;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < TMA_STAGES; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(empty + q)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(done)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    bool ok = true;

    // warp 0, lane 0: producer; warp 1, lane 0: MMA issuer.  The other lanes of those
    // two warps wait at __syncwarp, so they take no issue slots from the role lane
    // (spinning in the same warp on the accumulator barrier halved the pipeline).
    if (warp == 0) {
        if (lane == 0) {
        // producer: chunk kc = tap * nck + cc, A = input box shifted by the tap, B = weights
        for (int kc = 0; kc < nk && ok; ++kc) {
            const int st = kc % TMA_STAGES, use = kc / TMA_STAGES;
            if (use > 0 && !wait_parity(saddr(empty + st), (uint32_t)((use + 1) & 1))) ok = false;
            if (!ok) break;
            const int tap = kc / nck, cc = kc - tap * nck;
            const int sgn = MODE == 0 ? 1 : -1;
            const int dy = sgn * (tap / 3 - 1), dx = sgn * (tap % 3 - 1);
            const int c = cc * TK;
            const uint32_t a_dst = saddr(smem + st * STAGE_BYTES), b_dst = a_dst + A_BYTES;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(full + st)), "r"(kStageTx)
                         : "memory");
            if (c < C1) tma_load_4d(a_dst, &ta1, c, x0 + dx, y0 + dy, img, saddr(full + st));
            else tma_load_4d(a_dst, &ta2, c - C1, x0 + dx, y0 + dy, img, saddr(full + st));
            if (MODE == 0) tma_load_2d(b_dst, &tb, tap * (C1 + C2) + c, n0, saddr(full + st));
            else tma_load_3d(b_dst, &tb, c, n0, tap, saddr(full + st));
        }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
        // MMA issuer
        for (int kc = 0; kc < nk && ok; ++kc) {
            const int st = kc % TMA_STAGES, use = kc / TMA_STAGES;
            if (!wait_parity(saddr(full + st), (uint32_t)(use & 1))) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t a0 = saddr(smem + st * STAGE_BYTES), b0 = a0 + A_BYTES;
#pragma unroll
            for (int j = 0; j < TK / 16; ++j)
                mma_f16(tmem, smem_desc_sw128(a0 + 32 * j), smem_desc_sw128(b0 + 32 * j), kIdesc,
                        (kc > 0 || j > 0) ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             saddr(empty + st))
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(done))
                     : "memory");
        }
        __syncwarp();
    }
    // everyone: the accumulator is complete when `done` fires (the issuer commits it
    // even after a failed wait, so this wait ends)
    if (!wait_parity(saddr(done), 0u)) ok = false;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (__syncthreads_or(ok ? 0 : 1)) ok = false;
    if (ok) {
        const int p = m0 + warp * 32 + lane;  // TMEM lane = tile row = pixel
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
            if (MODE == 0) {
#pragma unroll
                for (int q = 0; q < 16; q += 2) {
                    const int col = n0 + c + q;
                    float v0 = __uint_as_float(r[q]) + bias[col], v1 = __uint_as_float(r[q + 1]) + bias[col + 1];
                    if (RELU) {
                        v0 = fmaxf(v0, 0.f);
                        v1 = fmaxf(v1, 0.f);
                    }
                    *(__nv_bfloat162*)(y + (size_t)p * Cout + col) = __floats2bfloat162_rn(v0, v1);
                }
            } else {
                // output channel tile n0 lies in [o1 | o2]: both channel counts are multiples of TN
                bf16* out = n0 < Cout ? y + (size_t)p * Cout + n0 : o2 + (size_t)p * Co2 + (n0 - Cout);
#pragma unroll
                for (int q = 0; q < 16; q += 2)
                    *(__nv_bfloat162*)(out + c + q) = __floats2bfloat162_rn(__uint_as_float(r[q]), __uint_as_float(r[q + 1]));
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
}


// ---------------------------------------------------------------------------
// Persistent form of k_conv_fwd_tma (same MODEs, operands, stage layout and MMA
// order per tile, so the same values bitwise): a CTA loops over output tiles
// (tile t = n-tile * m-tiles + m-tile, t += gridDim.x) with one operand ring that
// runs across tile boundaries and two accumulators in tensor memory, so the
// epilogue of one tile runs while the MMAs of the next are issued.  Warp 0 lane 0
// issues the TMA copies, warp 1 lane 0 the MMAs; warps 2-5 are the epilogue (warp w
// reads TMEM lanes 32 (w % 4) .. + 31).  Barriers: full / empty per stage, acc_full
// per accumulator (the MMAs of a tile committed), acc_empty per accumulator (the
// four epilogue warps have read it).  Every wait is bounded; a role that gives up
// records the error and stops, the others then run out their own bounded waits.
// ---------------------------------------------------------------------------
constexpr int P_THREADS = 192;
#ifndef GLNN_P_STAGES
#define GLNN_P_STAGES 3
#endif
constexpr int P_STAGES = GLNN_P_STAGES;  // operand stages of the persistent kernel (the ring runs across tiles)
constexpr int P_SMEM = P_STAGES * STAGE_BYTES + 1024 + (2 * P_STAGES + 4) * 8 + 16;
constexpr uint32_t kTmemColsP = 2 * TN;  // two FP32 accumulators of TN columns
static_assert(P_SMEM <= 227 * 1024, "persistent conv stages exceed shared memory");

template <int MODE, int RELU>
__global__ void __launch_bounds__(P_THREADS)
k_conv_tma_persist(const __grid_constant__ CUtensorMap ta1, const __grid_constant__ CUtensorMap ta2,
                   const __grid_constant__ CUtensorMap tb, const float* __restrict__ bias, bf16* __restrict__ y,
                   int Cout, bf16* __restrict__ o2, int Co2, int C1, int C2, int H, int W, int nmt, int ntiles,
                   int* err) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + P_STAGES * STAGE_BYTES);
    uint64_t* empty = full + P_STAGES;
    uint64_t* acc_full = empty + P_STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint32_t* tslot = (uint32_t*)(acc_empty + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nck = (C1 + C2) / TK, nk = 9 * nck;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                     "r"(kTmemColsP)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < P_STAGES; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(empty + q)) : "memory");
        }
        for (int q = 0; q < 2; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(acc_full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(saddr(acc_empty + q)) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {
            int g = 0;  // chunks issued by this CTA, across its tiles
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int m0 = (t % nmt) * TM, n0 = (t / nmt) * TN;
                const int img = m0 / (H * W), rem = m0 - img * H * W, y0 = rem / W, x0 = rem - y0 * W;
                for (int kc = 0; kc < nk; ++kc, ++g) {
                    const int st = g % P_STAGES, use = g / P_STAGES;
                    if (use > 0 && !wait_parity(saddr(empty + st), (uint32_t)((use + 1) & 1))) {
                        ok = false;
                        break;
                    }
                    const int tap = kc / nck, cc = kc - tap * nck;
                    const int sgn = MODE == 0 ? 1 : -1;
                    const int dy = sgn * (tap / 3 - 1), dx = sgn * (tap % 3 - 1);
                    const int c = cc * TK;
                    const uint32_t a_dst = saddr(smem + st * STAGE_BYTES), b_dst = a_dst + A_BYTES;
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(full + st)),
                                 "r"(kStageTx)
                                 : "memory");
                    if (c < C1) tma_load_4d(a_dst, &ta1, c, x0 + dx, y0 + dy, img, saddr(full + st));
                    else tma_load_4d(a_dst, &ta2, c - C1, x0 + dx, y0 + dy, img, saddr(full + st));
                    if (MODE == 0) tma_load_2d(b_dst, &tb, tap * (C1 + C2) + c, n0, saddr(full + st));
                    else tma_load_3d(b_dst, &tb, c, n0, tap, saddr(full + st));
                }
            }
            // copies still in flight land before the CTA leaves: wait (bounded) for the
            // last stages issued
            for (int q = 0; q < P_STAGES && q < g; ++q) {
                const int gg = g - 1 - q, st = gg % P_STAGES, use = gg / P_STAGES;
                wait_parity(saddr(full + st), (uint32_t)(use & 1));
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            int g = 0, lt = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++lt) {
                const int acc = lt & 1, ause = lt >> 1;
                if (ause > 0 && !wait_parity(saddr(acc_empty + acc), (uint32_t)((ause + 1) & 1))) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(acc * TN);
                for (int kc = 0; kc < nk; ++kc, ++g) {
                    const int st = g % P_STAGES, use = g / P_STAGES;
                    if (!wait_parity(saddr(full + st), (uint32_t)(use & 1))) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t a0 = saddr(smem + st * STAGE_BYTES), b0 = a0 + A_BYTES;
#pragma unroll
                    for (int j = 0; j < TK / 16; ++j)
                        mma_f16(d, smem_desc_sw128(a0 + 32 * j), smem_desc_sw128(b0 + 32 * j), kIdesc,
                                (kc > 0 || j > 0) ? 1u : 0u);
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     saddr(empty + st))
                                 : "memory");
                }
                // the tile's accumulator is complete once its MMAs are (committed even
                // after a failed wait, so the epilogue's wait ends)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 saddr(acc_full + acc))
                             : "memory");
            }
        }
        __syncwarp();
    } else {
        // epilogue warps 2..5: TMEM lane quarter w % 4
        const int quarter = warp & 3;
        int lt = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
            const int acc = lt & 1, ause = lt >> 1;
            const bool got = wait_parity(saddr(acc_full + acc), (uint32_t)(ause & 1));
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (!got) {
                ok = false;
                break;
            }
            const int m0 = (t % nmt) * TM, n0 = (t / nmt) * TN;
            const int p = m0 + quarter * 32 + lane;  // TMEM lane = tile row = pixel
#pragma unroll
            for (int c = 0; c < TN; c += 16) {
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                    : "r"(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * TN + c))
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (MODE == 0) {
#pragma unroll
                    for (int q = 0; q < 16; q += 2) {
                        const int col = n0 + c + q;
                        float v0 = __uint_as_float(r[q]) + bias[col], v1 = __uint_as_float(r[q + 1]) + bias[col + 1];
                        if (RELU) {
                            v0 = fmaxf(v0, 0.f);
                            v1 = fmaxf(v1, 0.f);
                        }
                        *(__nv_bfloat162*)(y + (size_t)p * Cout + col) = __floats2bfloat162_rn(v0, v1);
                    }
                } else {
                    bf16* out = n0 < Cout ? y + (size_t)p * Cout + n0 : o2 + (size_t)p * Co2 + (n0 - Cout);
#pragma unroll
                    for (int q = 0; q < 16; q += 2)
                        *(__nv_bfloat162*)(out + c + q) =
                            __floats2bfloat162_rn(__uint_as_float(r[q]), __uint_as_float(r[q + 1]));
                }
            }
            // this warp has read the accumulator: the MMAs of the tile after next may use it
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(acc_empty + acc)) : "memory");
        }
    }
    if (!ok) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemColsP) : "memory");
}

// ---------------------------------------------------------------------------
// k_conv_tma_persist with the B operand resident: a CTA works on one output-channel
// tile (n-tile = blockIdx.x % NT) and loops over pixel tiles; it loads the n-tile's
// weights (all 9 taps x input-channel chunks, 8 KB each) into shared memory once,
// and only the shifted activation boxes (16 KB per chunk) stream through the ring.
// This removes the weight re-reads, a third of the bytes that move from L2 into the
// SMs.  Used when the weights of an n-tile fit (at most two 64-channel input
// chunks); the same MMAs in the same order, so the same values bitwise.
// ---------------------------------------------------------------------------
constexpr int BR_MAX_CHUNKS = 18;  // 9 taps x 2 input-channel chunks
__host__ __device__ constexpr int br_smem_bytes(int nk) {
    return P_STAGES * A_BYTES + nk * B_BYTES + 1024 + (2 * P_STAGES + 5) * 8 + 16;
}
static_assert(br_smem_bytes(BR_MAX_CHUNKS) <= 227 * 1024, "resident-weight conv exceeds shared memory");

template <int MODE, int RELU>
__global__ void __launch_bounds__(P_THREADS)
k_conv_tma_bres(const __grid_constant__ CUtensorMap ta1, const __grid_constant__ CUtensorMap ta2,
                const __grid_constant__ CUtensorMap tb, const float* __restrict__ bias, bf16* __restrict__ y, int Cout,
                bf16* __restrict__ o2, int Co2, int C1, int C2, int H, int W, int nmt, int NT, int* err) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int nck = (C1 + C2) / TK, nk = 9 * nck;
    unsigned char* bres = smem + P_STAGES * A_BYTES;
    uint64_t* full = (uint64_t*)(bres + nk * B_BYTES);
    uint64_t* empty = full + P_STAGES;
    uint64_t* acc_full = empty + P_STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* b_full = acc_empty + 2;
    uint32_t* tslot = (uint32_t*)(b_full + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int cpn = gridDim.x / NT;  // CTAs per n-tile
    const int nt = blockIdx.x % NT, mt0 = blockIdx.x / NT, n0 = nt * TN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                     "r"(kTmemColsP)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < P_STAGES; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(empty + q)) : "memory");
        }
        for (int q = 0; q < 2; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(acc_full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(saddr(acc_empty + q)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(b_full)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {
            // the n-tile's weights, once
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(b_full)),
                         "r"((uint32_t)(nk * B_BYTES))
                         : "memory");
            for (int kc = 0; kc < nk; ++kc) {
                const int tap = kc / nck, c = (kc - tap * nck) * TK;
                const uint32_t b_dst = saddr(bres + kc * B_BYTES);
                if (MODE == 0) tma_load_2d(b_dst, &tb, tap * (C1 + C2) + c, n0, saddr(b_full));
                else tma_load_3d(b_dst, &tb, c, n0, tap, saddr(b_full));
            }
            int g = 0;
            for (int mt = mt0; mt < nmt && ok; mt += cpn) {
                const int m0 = mt * TM;
                const int img = m0 / (H * W), rem = m0 - img * H * W, y0 = rem / W, x0 = rem - y0 * W;
                for (int kc = 0; kc < nk; ++kc, ++g) {
                    const int st = g % P_STAGES, use = g / P_STAGES;
                    if (use > 0 && !wait_parity(saddr(empty + st), (uint32_t)((use + 1) & 1))) {
                        ok = false;
                        break;
                    }
                    const int tap = kc / nck, cc = kc - tap * nck;
                    const int sgn = MODE == 0 ? 1 : -1;
                    const int dy = sgn * (tap / 3 - 1), dx = sgn * (tap % 3 - 1);
                    const int c = cc * TK;
                    const uint32_t a_dst = saddr(smem + st * A_BYTES);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(full + st)),
                                 "r"((uint32_t)A_BYTES)
                                 : "memory");
                    if (c < C1) tma_load_4d(a_dst, &ta1, c, x0 + dx, y0 + dy, img, saddr(full + st));
                    else tma_load_4d(a_dst, &ta2, c - C1, x0 + dx, y0 + dy, img, saddr(full + st));
                }
            }
            // copies still in flight land before the CTA leaves (bounded waits)
            wait_parity(saddr(b_full), 0u);
            for (int q = 0; q < P_STAGES && q < g; ++q) {
                const int gg = g - 1 - q, st = gg % P_STAGES, use = gg / P_STAGES;
                wait_parity(saddr(full + st), (uint32_t)(use & 1));
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            if (!wait_parity(saddr(b_full), 0u)) ok = false;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            int g = 0, lt = 0;
            for (int mt = mt0; mt < nmt && ok; mt += cpn, ++lt) {
                const int acc = lt & 1, ause = lt >> 1;
                if (ause > 0 && !wait_parity(saddr(acc_empty + acc), (uint32_t)((ause + 1) & 1))) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(acc * TN);
                for (int kc = 0; kc < nk; ++kc, ++g) {
                    const int st = g % P_STAGES, use = g / P_STAGES;
                    if (!wait_parity(saddr(full + st), (uint32_t)(use & 1))) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t a0 = saddr(smem + st * A_BYTES), b0 = saddr(bres + kc * B_BYTES);
#pragma unroll
                    for (int j = 0; j < TK / 16; ++j)
                        mma_f16(d, smem_desc_sw128(a0 + 32 * j), smem_desc_sw128(b0 + 32 * j), kIdesc,
                                (kc > 0 || j > 0) ? 1u : 0u);
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     saddr(empty + st))
                                 : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 saddr(acc_full + acc))
                             : "memory");
            }
        }
        __syncwarp();
    } else {
        const int quarter = warp & 3;
        int lt = 0;
        for (int mt = mt0; mt < nmt; mt += cpn, ++lt) {
            const int acc = lt & 1, ause = lt >> 1;
            const bool got = wait_parity(saddr(acc_full + acc), (uint32_t)(ause & 1));
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (!got) {
                ok = false;
                break;
            }
            const int p = mt * TM + quarter * 32 + lane;
#pragma unroll
            for (int c = 0; c < TN; c += 16) {
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                    : "r"(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * TN + c))
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (MODE == 0) {
#pragma unroll
                    for (int q = 0; q < 16; q += 2) {
                        const int col = n0 + c + q;
                        float v0 = __uint_as_float(r[q]) + bias[col], v1 = __uint_as_float(r[q + 1]) + bias[col + 1];
                        if (RELU) {
                            v0 = fmaxf(v0, 0.f);
                            v1 = fmaxf(v1, 0.f);
                        }
                        *(__nv_bfloat162*)(y + (size_t)p * Cout + col) = __floats2bfloat162_rn(v0, v1);
                    }
                } else {
                    bf16* out = n0 < Cout ? y + (size_t)p * Cout + n0 : o2 + (size_t)p * Co2 + (n0 - Cout);
#pragma unroll
                    for (int q = 0; q < 16; q += 2)
                        *(__nv_bfloat162*)(out + c + q) =
                            __floats2bfloat162_rn(__uint_as_float(r[q]), __uint_as_float(r[q + 1]));
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(acc_empty + acc)) : "memory");
        }
    }
    if (!ok) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemColsP) : "memory");
}

// ---------------------------------------------------------------------------
// k_conv_tma_bres with each input row loaded once: for 128-pixel tiles that lie in
// one image row (w a multiple of 128), a stage holds one tap row dy of the tile, i.e.
// for every input-channel chunk one box of 130 pixels (the tile and a one-pixel halo
// on each side, zeros outside the image) x 64 channels.  The three taps dx of that row
// read the same box from pixel 0, 1 or 2: the A descriptor starts 0, 128 or 256 bytes
// into the 1024-byte swizzle atom (see smem_desc_sw128_at).  The activation bytes
// moved from L2 per tile fall from 9 x 16 KB to 3 x 16.25 KB per channel chunk.  The
// MMAs run in the order of the other kernels (tap-major, channel chunk inner), so
// the results are the same bitwise.
// ---------------------------------------------------------------------------
constexpr int HALO_PX = TM + 2;                        // 130 pixels per box
constexpr int HALO_BOX = HALO_PX * TK * 2;             // 16,640 bytes
constexpr int HALO_SLOT = 17 * 1024;                   // a box's 1024-aligned slot
__host__ __device__ constexpr int halo_stages(int nck) { return nck == 1 ? 3 : 2; }
__host__ __device__ constexpr int halo_smem_bytes(int nck) {
    return halo_stages(nck) * nck * HALO_SLOT + 9 * nck * B_BYTES + 1024 + (2 * 3 + 5) * 8 + 16;
}
static_assert(halo_smem_bytes(1) <= 227 * 1024 && halo_smem_bytes(2) <= 227 * 1024, "halo conv exceeds shared memory");

// A view starting 128 or 256 bytes into a swizzle atom: the MMA applies the 128-byte
// swizzle by the absolute shared-memory address bits, as the TMA copy that wrote the
// box did, so the descriptor is the plain one (its base-offset field stays 0; set to
// (start >> 7) & 7 it gave wrong products, measured).
__device__ __forceinline__ uint64_t smem_desc_sw128_at(uint32_t start) { return smem_desc_sw128(start); }

template <int MODE, int RELU>
__global__ void __launch_bounds__(P_THREADS)
k_conv_tma_halo(const __grid_constant__ CUtensorMap ta1, const __grid_constant__ CUtensorMap ta2,
                const __grid_constant__ CUtensorMap tb, const float* __restrict__ bias, bf16* __restrict__ y, int Cout,
                bf16* __restrict__ o2, int Co2, int C1, int C2, int H, int W, int nmt, int NT, int* err) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int nck = (C1 + C2) / TK, nk = 9 * nck, S = halo_stages(nck);
    const int stage_bytes = nck * HALO_SLOT;
    unsigned char* bres = smem + S * stage_bytes;
    uint64_t* full = (uint64_t*)(bres + nk * B_BYTES);
    uint64_t* empty = full + 3;
    uint64_t* acc_full = empty + 3;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* b_full = acc_empty + 2;
    uint32_t* tslot = (uint32_t*)(b_full + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int cpn = gridDim.x / NT;
    const int nt = blockIdx.x % NT, mt0 = blockIdx.x / NT, n0 = nt * TN;
    const int sgn = MODE == 0 ? 1 : -1;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                     "r"(kTmemColsP)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < S; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(empty + q)) : "memory");
        }
        for (int q = 0; q < 2; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(acc_full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(saddr(acc_empty + q)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(b_full)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(b_full)),
                         "r"((uint32_t)(nk * B_BYTES))
                         : "memory");
            for (int kc = 0; kc < nk; ++kc) {
                const int tap = kc / nck, c = (kc - tap * nck) * TK;
                const uint32_t b_dst = saddr(bres + kc * B_BYTES);
                if (MODE == 0) tma_load_2d(b_dst, &tb, tap * (C1 + C2) + c, n0, saddr(b_full));
                else tma_load_3d(b_dst, &tb, c, n0, tap, saddr(b_full));
            }
            int g = 0;  // stages filled, across tiles
            for (int mt = mt0; mt < nmt && ok; mt += cpn) {
                const int m0 = mt * TM;
                const int img = m0 / (H * W), rem = m0 - img * H * W, y0 = rem / W, x0 = rem - y0 * W;
                for (int ty = 0; ty < 3; ++ty, ++g) {
                    const int st = g % S, use = g / S;
                    if (use > 0 && !wait_parity(saddr(empty + st), (uint32_t)((use + 1) & 1))) {
                        ok = false;
                        break;
                    }
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(full + st)),
                                 "r"((uint32_t)(nck * HALO_BOX))
                                 : "memory");
                    const int yy = y0 + sgn * (ty - 1);
                    for (int cc = 0; cc < nck; ++cc) {
                        const int c = cc * TK;
                        const uint32_t dst = saddr(smem + st * stage_bytes + cc * HALO_SLOT);
                        if (c < C1) tma_load_4d(dst, &ta1, c, x0 - 1, yy, img, saddr(full + st));
                        else tma_load_4d(dst, &ta2, c - C1, x0 - 1, yy, img, saddr(full + st));
                    }
                }
            }
            wait_parity(saddr(b_full), 0u);
            for (int q = 0; q < S && q < g; ++q) {
                const int gg = g - 1 - q, st = gg % S, use = gg / S;
                wait_parity(saddr(full + st), (uint32_t)(use & 1));
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            if (!wait_parity(saddr(b_full), 0u)) ok = false;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            int g = 0, lt = 0;
            for (int mt = mt0; mt < nmt && ok; mt += cpn, ++lt) {
                const int acc = lt & 1, ause = lt >> 1;
                if (ause > 0 && !wait_parity(saddr(acc_empty + acc), (uint32_t)((ause + 1) & 1))) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(acc * TN);
                for (int ty = 0; ty < 3; ++ty, ++g) {
                    const int st = g % S, use = g / S;
                    if (!wait_parity(saddr(full + st), (uint32_t)(use & 1))) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    for (int tx = 0; tx < 3; ++tx) {
                        // pixel offset of the view in the box: +tx-1 (forward) or -(tx-1) (data gradient)
                        const int off = MODE == 0 ? tx : 2 - tx;
                        for (int cc = 0; cc < nck; ++cc) {
                            const int kc = (ty * 3 + tx) * nck + cc;
                            const uint32_t a0 = saddr(smem + st * stage_bytes + cc * HALO_SLOT) + 128u * off;
                            const uint32_t b0 = saddr(bres + kc * B_BYTES);
#pragma unroll
                            for (int j = 0; j < TK / 16; ++j)
                                mma_f16(d, smem_desc_sw128_at(a0 + 32 * j), smem_desc_sw128(b0 + 32 * j), kIdesc,
                                        (kc > 0 || j > 0) ? 1u : 0u);
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     saddr(empty + st))
                                 : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 saddr(acc_full + acc))
                             : "memory");
            }
        }
        __syncwarp();
    } else {
        const int quarter = warp & 3;
        int lt = 0;
        for (int mt = mt0; mt < nmt; mt += cpn, ++lt) {
            const int acc = lt & 1, ause = lt >> 1;
            const bool got = wait_parity(saddr(acc_full + acc), (uint32_t)(ause & 1));
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (!got) {
                ok = false;
                break;
            }
            const int p = mt * TM + quarter * 32 + lane;
#pragma unroll
            for (int c = 0; c < TN; c += 16) {
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                    : "r"(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * TN + c))
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (MODE == 0) {
#pragma unroll
                    for (int q = 0; q < 16; q += 2) {
                        const int col = n0 + c + q;
                        float v0 = __uint_as_float(r[q]) + bias[col], v1 = __uint_as_float(r[q + 1]) + bias[col + 1];
                        if (RELU) {
                            v0 = fmaxf(v0, 0.f);
                            v1 = fmaxf(v1, 0.f);
                        }
                        *(__nv_bfloat162*)(y + (size_t)p * Cout + col) = __floats2bfloat162_rn(v0, v1);
                    }
                } else {
                    bf16* out = n0 < Cout ? y + (size_t)p * Cout + n0 : o2 + (size_t)p * Co2 + (n0 - Cout);
#pragma unroll
                    for (int q = 0; q < 16; q += 2)
                        *(__nv_bfloat162*)(out + c + q) =
                            __floats2bfloat162_rn(__uint_as_float(r[q]), __uint_as_float(r[q + 1]));
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(acc_empty + acc)) : "memory");
        }
    }
    if (!ok) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemColsP) : "memory");
}

// ---------------------------------------------------------------------------
// Weight gradient on tcgen05 with TMA operands: dW[co][tap][ci] =
// sum_p dy'[p][co] x[p + off(tap)][ci] (dy' = dy * relu'(y), formed by
// k_relu_mask_dy beforehand), as D[m][co] = sum_k A[m][k] B[k][co] with
// M = 128 rows = (two taps, 64 input channels), N = 64 output channels and
// K = pixels.  A K chunk of 64 pixels is three boxes of the 4-D activation
// tensors, each 64 pixels x 64 channels: the input shifted by the pair's first
// tap, the input shifted by its second tap, and dy'.  They land as pixel rows of
// 128 bytes (64 channels) with the 128-byte swizzle, which is the MN-major
// operand layout (M, resp. N, contiguous within a row; K = the row index): both
// operands are MN-major in the instruction descriptor, the two tap boxes are the
// two 64-row atoms of A along M (leading byte offset 8 KB), 8-row groups along K
// are 1024 bytes apart, and a K step of 16 pixels advances the start by 2 KB.
// Tap pairs (0,1) (2,3) (4,5) (6,7) (8,-): the last pair's second half is not
// stored.  The pixel range is split over blockIdx.y (split-K); every CTA writes
// its tile of partial sums to ws[split][co][tap][ci], which k_sum_splits reduces
// in a fixed order.  Thread 0 issues the copies into a 4-stage ring, thread 32
// the MMAs; every wait is bounded, and a CTA whose wait ran out writes NaN
// partials (and sets *err), so the failure reaches dW.
// ---------------------------------------------------------------------------
constexpr int WG_PX = 64;                          // pixels per K chunk
constexpr int WG_BOX = WG_PX * 64 * 2;             // one 64 x 64 bf16 box: 8 KB
constexpr int WG_STAGE = 3 * WG_BOX;               // two tap boxes + dy': 24 KB
#ifndef GLNN_WG_STAGES
#define GLNN_WG_STAGES 3
#endif
constexpr int WG_STAGES = GLNN_WG_STAGES;
constexpr int WG_SMEM = WG_STAGES * WG_STAGE + 1024 + (2 * WG_STAGES + 2) * 8;
static_assert(WG_STAGES >= 1 && WG_SMEM <= 227 * 1024, "weight-gradient stages exceed shared memory");
// kIdesc (M = 128, N = 64, bf16 -> f32) with A and B MN-major (bits 15, 16)
constexpr uint32_t kIdescMN = kIdesc | (1u << 15) | (1u << 16);

// SM100 shared-memory matrix descriptor, MN-major with the 128-byte swizzle:
// leading byte offset = distance between 64-element atoms along M or N, stride
// byte offset = distance between 8-row groups along K (1024 B here).
__device__ __forceinline__ uint64_t smem_desc_sw128_mn(uint32_t start, uint32_t lbo) {
    uint64_t d = (uint64_t)((start >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

__global__ void __launch_bounds__(NTH)
k_conv_wgrad_tma(const __grid_constant__ CUtensorMap tx1, const __grid_constant__ CUtensorMap tx2,
                 const __grid_constant__ CUtensorMap tdy, float* __restrict__ ws, int C1, int C2, int Cout, int H,
                 int W, int P, int chunk, int* err) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* full = (uint64_t*)(smem + WG_STAGES * WG_STAGE);
    uint64_t* empty = full + WG_STAGES;
    uint64_t* done = empty + WG_STAGES;
    uint32_t* tslot = (uint32_t*)(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Cin = C1 + C2, nco = Cout / 64, nci = Cin / 64;
    int t = blockIdx.x;
    const int oc = t % nco;
    t /= nco;
    const int cc = t % nci, g = t / nci;  // input-channel chunk, tap pair
    const int tap0 = 2 * g, tap1 = g < 4 ? 2 * g + 1 : 8;
    const int pbeg = blockIdx.y * chunk, pend = min(P, pbeg + chunk);
    const int nk = pend > pbeg ? (pend - pbeg) / WG_PX : 0;
    const int c = cc * 64;
    const CUtensorMap* xm = c < C1 ? &tx1 : &tx2;
    const int cx = c < C1 ? c : c - C1;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(tslot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        for (int q = 0; q < WG_STAGES; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(full + q)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(empty + q)) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(saddr(done)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (nk > 0) {
        // warp 0, lane 0: producer; warp 1, lane 0: MMA issuer; their other lanes wait
        // at __syncwarp (as in k_conv_fwd_tma)
        if (warp == 0) {
            if (lane == 0) {
            const int dy0 = tap0 / 3 - 1, dx0 = tap0 % 3 - 1, dy1 = tap1 / 3 - 1, dx1 = tap1 % 3 - 1;
            for (int kc = 0; kc < nk && ok; ++kc) {
                const int st = kc % WG_STAGES, use = kc / WG_STAGES;
                if (use > 0 && !wait_parity(saddr(empty + st), (uint32_t)((use + 1) & 1))) ok = false;
                if (!ok) break;
                const int p0 = pbeg + kc * WG_PX;
                const int img = p0 / (H * W), rem = p0 - img * H * W, y0 = rem / W, x0 = rem - y0 * W;
                const uint32_t dst = saddr(smem + st * WG_STAGE);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(full + st)),
                             "r"((uint32_t)WG_STAGE)
                             : "memory");
                tma_load_4d(dst, xm, cx, x0 + dx0, y0 + dy0, img, saddr(full + st));
                tma_load_4d(dst + WG_BOX, xm, cx, x0 + dx1, y0 + dy1, img, saddr(full + st));
                tma_load_4d(dst + 2 * WG_BOX, &tdy, oc * 64, x0, y0, img, saddr(full + st));
            }
            }
            __syncwarp();
        } else if (warp == 1) {
            if (lane == 0) {
            for (int kc = 0; kc < nk && ok; ++kc) {
                const int st = kc % WG_STAGES, use = kc / WG_STAGES;
                if (!wait_parity(saddr(full + st), (uint32_t)(use & 1))) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t a0 = saddr(smem + st * WG_STAGE), b0 = a0 + 2 * WG_BOX;
#pragma unroll
                for (int j = 0; j < WG_PX / 16; ++j)
                    mma_f16(tmem, smem_desc_sw128_mn(a0 + 2048 * j, WG_BOX), smem_desc_sw128_mn(b0 + 2048 * j, WG_BOX),
                            kIdescMN, (kc > 0 || j > 0) ? 1u : 0u);
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 saddr(empty + st))
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             saddr(done))
                         : "memory");
            }
            __syncwarp();
        }
        if (!wait_parity(saddr(done), 0u)) ok = false;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    }
    if (__syncthreads_or(ok ? 0 : 1)) ok = false;
    // TMEM lane m = warp * 32 + lane: tap (m < 64 ? tap0 : tap1), input channel c + m % 64
    const int m = warp * 32 + lane;
    const int tap = m < 64 ? tap0 : tap1;
    const bool store = m < 64 || g < 4;
    float* out = ws + (size_t)blockIdx.y * Cout * 9 * Cin + (size_t)tap * Cin + c + (m & 63);
#pragma unroll
    for (int col = 0; col < 64; col += 16) {
        uint32_t r[16];
        if (nk > 0) {
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)col)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        } else {
#pragma unroll
            for (int q = 0; q < 16; ++q) r[q] = 0u;
        }
        if (store) {
#pragma unroll
            for (int q = 0; q < 16; ++q)
                out[(size_t)(oc * 64 + col + q) * 9 * Cin] = ok ? __uint_as_float(r[q]) : __int_as_float(0x7fc00000);
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// dy' = dy * (y > 0), 8 bf16 per thread step
__global__ void k_relu_mask_dy(const uint4* __restrict__ dy, const uint4* __restrict__ y, uint4* __restrict__ out,
                               long long n8) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n8; i += (long long)gridDim.x * blockDim.x) {
        const uint4 d = dy[i], v = y[i];
        out[i] = make_uint4(relu_mask2(d.x, v.x), relu_mask2(d.y, v.y), relu_mask2(d.z, v.z), relu_mask2(d.w, v.w));
    }
}

}  // namespace glnn_tc

using namespace glnn_tc;

// The kernels use more than the default 48 KB of dynamic shared memory.
template <int MODE, int RELU> static cudaError_t conv_tc_smem_attr() {
    static cudaError_t e = cudaFuncSetAttribute(k_conv_tc<MODE, RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                SMEM_BYTES);
    return e;
}

// --- TMA forward: tensor maps and the shapes it takes -------------------------
static int g_conv_tma = 2;  // glnn_set_conv_tma: 0 thread gather, 1 TMA per tile, 2 TMA persistent

static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// activations [n][h][w][c] (bf16), box = 64 channels x one tile of `px` pixels
// (whole rows or a run of one row)
static bool act_map(CUtensorMap* m, const void* base, int c, int n, int h, int w, int px = TM) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
    if (!enc) return false;
    const int wb = w < px ? w : px, hb = px / wb;
    cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2};
    cuuint32_t box[4] = {(cuuint32_t)TK, (cuuint32_t)wb, (cuuint32_t)hb, 1u};
    cuuint32_t es[4] = {1u, 1u, 1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// activations [n][h][w][c] (bf16), box = 64 channels x 130 pixels of one row (a
// 128-pixel tile with a one-pixel halo on each side)
static bool act_map_halo(CUtensorMap* m, const void* base, int c, int n, int h, int w) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
    if (!enc) return false;
    cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2};
    cuuint32_t box[4] = {(cuuint32_t)TK, (cuuint32_t)HALO_PX, 1u, 1u};
    cuuint32_t es[4] = {1u, 1u, 1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// weights [rows][k] (bf16, k contiguous), box = 64 k x 64 rows
static bool weight_map(CUtensorMap* m, const void* base, long long k, long long rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)k * 2};
    cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)TN};
    cuuint32_t es[2] = {1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the shapes the TMA forward takes: 64-channel chunks, 64-channel output tiles,
// 128-pixel tiles that are whole rows or whole groups of rows of one image
static bool conv_tma_shape_ok(int c1, int c2, int h, int w, int cout) {
    return c1 % TK == 0 && c2 % TK == 0 && cout % TN == 0 && ((long long)h * w) % TM == 0 && (w % TM == 0 || TM % w == 0);
}

template <int MODE, int RELU> static cudaError_t conv_tma_smem_attr() {
    static cudaError_t e =
        cudaFuncSetAttribute(k_conv_fwd_tma<MODE, RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize, TMA_SMEM);
    return e;
}

// Wt [9][cin][cout] (bf16, cout contiguous), box = 64 cout x 64 cin x one tap
static bool weight_t_map(CUtensorMap* m, const void* base, int cin, int cout) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)cout, (cuuint64_t)cin, 9u};
    cuuint64_t strides[2] = {(cuuint64_t)cout * 2, (cuuint64_t)cin * cout * 2};
    cuuint32_t box[3] = {(cuuint32_t)TK, (cuuint32_t)TN, 1u};
    cuuint32_t es[3] = {1u, 1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int MODE, int RELU> static cudaError_t conv_persist_smem_attr() {
    static cudaError_t e =
        cudaFuncSetAttribute(k_conv_tma_persist<MODE, RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize, P_SMEM);
    return e;
}

template <int MODE, int RELU> static cudaError_t conv_bres_smem_attr() {
    static cudaError_t e = cudaFuncSetAttribute(k_conv_tma_bres<MODE, RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                br_smem_bytes(BR_MAX_CHUNKS));
    return e;
}

template <int MODE, int RELU> static cudaError_t conv_halo_smem_attr() {
    static cudaError_t e = cudaFuncSetAttribute(k_conv_tma_halo<MODE, RELU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                halo_smem_bytes(2));
    return e;
}
template <int MODE, int RELU> static int halo_grid(int NT, int nmt, int smem) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_conv_tma_halo<MODE, RELU>, P_THREADS, smem);
    int cpn = (sms > 0 ? sms : 152) * (per > 0 ? per : 1) / NT;
    cpn = cpn < 1 ? 1 : (cpn > nmt ? nmt : cpn);
    return NT * cpn;
}
// the halo kernel takes 128-pixel tiles inside one image row and at most two input chunks
static bool halo_ok(int w, int nck) { return g_conv_tma == 2 && w % TM == 0 && nck >= 1 && nck <= 2; }

// grid of the resident-weight kernel: NT x (CTAs per n-tile), the CTAs that fit on
// all SMs at this shared-memory size, at most one per pixel tile of an n-tile
template <int MODE, int RELU> static int bres_grid(int NT, int nmt, int smem) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_conv_tma_bres<MODE, RELU>, P_THREADS, smem);
    int cpn = (sms > 0 ? sms : 152) * (per > 0 ? per : 1) / NT;
    cpn = cpn < 1 ? 1 : (cpn > nmt ? nmt : cpn);
    return NT * cpn;
}

// grid of the persistent kernel: its resident CTAs on every SM, at most one per tile
static int persist_grid(int ntiles) {
    static int ctas = 0;
    if (!ctas) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        conv_persist_smem_attr<0, 0>();  // the occupancy query needs the kernel's shared-memory limit raised
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_conv_tma_persist<0, 0>, P_THREADS, P_SMEM);
        ctas = (sms > 0 ? sms : 152) * (per > 0 ? per : 1);
    }
    return ntiles < ctas ? ntiles : ctas;
}

// data gradient without a ReLU derivative (dy already masked) by TMA: 1 launched, 0 not taken
static int conv_bwd_data_tma(const void* dy, const void* wt, void* dx1, int c1, void* dx2, int c2, int n, int h, int w,
                             int cout, int* err, cudaStream_t s) {
    if (!g_conv_tma || !conv_tma_shape_ok(c1, c2, h, w, cout)) return 0;
    CUtensorMap ta, tb;
    if (!act_map(&ta, dy, cout, n, h, w) || !weight_t_map(&tb, wt, c1 + c2, cout)) return 0;
    const long long P = (long long)n * h * w;
    if (halo_ok(w, cout / TK)) {
        CUtensorMap th;
        if (!act_map_halo(&th, dy, cout, n, h, w) || conv_halo_smem_attr<1, 0>() != cudaSuccess) return 0;
        const int nmt = (int)(P / TM), NT = (c1 + c2) / TN, smem = halo_smem_bytes(cout / TK);
        k_conv_tma_halo<1, 0><<<halo_grid<1, 0>(NT, nmt, smem), P_THREADS, smem, s>>>(
            th, th, tb, nullptr, (bf16*)dx1, c1, (bf16*)dx2, c2, cout, 0, h, w, nmt, NT, err);
        return 1;
    }
    if (g_conv_tma == 2 && 9 * (cout / TK) <= BR_MAX_CHUNKS) {
        if (conv_bres_smem_attr<1, 0>() != cudaSuccess) return 0;
        const int nmt = (int)(P / TM), NT = (c1 + c2) / TN, smem = br_smem_bytes(9 * (cout / TK));
        k_conv_tma_bres<1, 0><<<bres_grid<1, 0>(NT, nmt, smem), P_THREADS, smem, s>>>(
            ta, ta, tb, nullptr, (bf16*)dx1, c1, (bf16*)dx2, c2, cout, 0, h, w, nmt, NT, err);
        return 1;
    }
    if (g_conv_tma == 2) {
        if (conv_persist_smem_attr<1, 0>() != cudaSuccess) return 0;
        const int nmt = (int)(P / TM), ntiles = nmt * ((c1 + c2) / TN);
        k_conv_tma_persist<1, 0><<<persist_grid(ntiles), P_THREADS, P_SMEM, s>>>(
            ta, ta, tb, nullptr, (bf16*)dx1, c1, (bf16*)dx2, c2, cout, 0, h, w, nmt, ntiles, err);
        return 1;
    }
    if (conv_tma_smem_attr<1, 0>() != cudaSuccess) return 0;
    dim3 grid((unsigned)(P / TM), (unsigned)((c1 + c2) / TN));
    k_conv_fwd_tma<1, 0><<<grid, NTH, TMA_SMEM, s>>>(ta, ta, tb, nullptr, (bf16*)dx1, c1, (bf16*)dx2, c2, cout, 0, h, w,
                                                     err);
    return 1;
}

// 1: launched; 0: shape or tensor maps not available (the caller uses the gather kernel)
static int conv_fwd_tma(const void* x1, int c1, const void* x2, int c2, const void* wb, const float* bias, void* y, int n,
                        int h, int w, int cout, int relu, int* err, cudaStream_t s) {
    if (!g_conv_tma || !conv_tma_shape_ok(c1, c2, h, w, cout)) return 0;
    CUtensorMap t1, t2, tb;
    if (!act_map(&t1, x1, c1, n, h, w)) return 0;
    if (c2 > 0) {
        if (!act_map(&t2, x2, c2, n, h, w)) return 0;
    } else {
        t2 = t1;
    }
    if (!weight_map(&tb, wb, 9LL * (c1 + c2), cout)) return 0;
    const long long P = (long long)n * h * w;
    if (halo_ok(w, (c1 + c2) / TK)) {
        CUtensorMap h1, h2;
        if (!act_map_halo(&h1, x1, c1, n, h, w)) return 0;
        if (c2 > 0) {
            if (!act_map_halo(&h2, x2, c2, n, h, w)) return 0;
        } else {
            h2 = h1;
        }
        if ((relu ? conv_halo_smem_attr<0, 1>() : conv_halo_smem_attr<0, 0>()) != cudaSuccess) return 0;
        const int nmt = (int)(P / TM), NT = cout / TN, smem = halo_smem_bytes((c1 + c2) / TK);
        if (relu)
            k_conv_tma_halo<0, 1><<<halo_grid<0, 1>(NT, nmt, smem), P_THREADS, smem, s>>>(
                h1, h2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2, h, w, nmt, NT, err);
        else
            k_conv_tma_halo<0, 0><<<halo_grid<0, 0>(NT, nmt, smem), P_THREADS, smem, s>>>(
                h1, h2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2, h, w, nmt, NT, err);
        return 1;
    }
    if (g_conv_tma == 2 && 9 * ((c1 + c2) / TK) <= BR_MAX_CHUNKS) {
        if ((relu ? conv_bres_smem_attr<0, 1>() : conv_bres_smem_attr<0, 0>()) != cudaSuccess) return 0;
        const int nmt = (int)(P / TM), NT = cout / TN, smem = br_smem_bytes(9 * ((c1 + c2) / TK));
        if (relu)
            k_conv_tma_bres<0, 1><<<bres_grid<0, 1>(NT, nmt, smem), P_THREADS, smem, s>>>(
                t1, t2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2, h, w, nmt, NT, err);
        else
            k_conv_tma_bres<0, 0><<<bres_grid<0, 0>(NT, nmt, smem), P_THREADS, smem, s>>>(
                t1, t2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2, h, w, nmt, NT, err);
        return 1;
    }
    if (g_conv_tma == 2) {
        if ((relu ? conv_persist_smem_attr<0, 1>() : conv_persist_smem_attr<0, 0>()) != cudaSuccess) return 0;
        const int nmt = (int)(P / TM), ntiles = nmt * (cout / TN);
        const int gs = persist_grid(ntiles);
        if (relu)
            k_conv_tma_persist<0, 1><<<gs, P_THREADS, P_SMEM, s>>>(t1, t2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2,
                                                                   h, w, nmt, ntiles, err);
        else
            k_conv_tma_persist<0, 0><<<gs, P_THREADS, P_SMEM, s>>>(t1, t2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2,
                                                                   h, w, nmt, ntiles, err);
        return 1;
    }
    if ((relu ? conv_tma_smem_attr<0, 1>() : conv_tma_smem_attr<0, 0>()) != cudaSuccess) return 0;
    dim3 grid((unsigned)(P / TM), (unsigned)(cout / TN));
    if (relu)
        k_conv_fwd_tma<0, 1><<<grid, NTH, TMA_SMEM, s>>>(t1, t2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2, h, w, err);
    else
        k_conv_fwd_tma<0, 0><<<grid, NTH, TMA_SMEM, s>>>(t1, t2, tb, bias, (bf16*)y, cout, nullptr, 0, c1, c2, h, w, err);
    return 1;
}

// --- weight gradient on tcgen05 -----------------------------------------------
// the shapes it takes: 64-channel chunks in and out, 64-pixel chunks that are runs
// of one row (w a multiple of 64) or whole groups of rows (64 a multiple of w)
static bool wgrad_tma_shape_ok(int c1, int c2, int h, int w, int cout) {
    return c1 % 64 == 0 && c2 % 64 == 0 && cout % 64 == 0 && ((long long)h * w) % WG_PX == 0 &&
           (w % WG_PX == 0 || WG_PX % w == 0);
}

// split-K plan: splits of whole 64-pixel chunks, about two CTAs per SM in all
void glnn_tc_wgrad_plan(int n, int h, int w, int cin, int cout, int* nz, int* chunk) {
    const long long P = (long long)n * h * w;
    const long long tiles = 5LL * (cin / 64) * (cout / 64);
    const long long nchunks = (P + WG_PX - 1) / WG_PX;
    long long z = (2 * 152 + tiles - 1) / tiles;
    z = z < 1 ? 1 : (z > nchunks ? nchunks : z);
    const long long per = (nchunks + z - 1) / z;
    *chunk = (int)(per * WG_PX);
    *nz = (int)((P + *chunk - 1) / *chunk);
}

// 1: launched (dy' and the partial sums enqueued on s); 0: shape, tensor maps or
// the switch rule it out (the caller runs the mma kernel)
int glnn_tc_wgrad(const void* dy, const void* y, int relu, const void* x1, int c1, const void* x2, int c2, float* ws,
                  void* dy_masked, int n, int h, int w, int cout, int* err, cudaStream_t s) {
    if (!g_conv_tma || !err || !wgrad_tma_shape_ok(c1, c2, h, w, cout)) return 0;
    const long long P = (long long)n * h * w;
    const void* dsrc = dy;
    if (relu) {
        if (!dy_masked) return 0;
        const long long n8 = P * cout / 8;
        const long long blocks = (n8 + 255) / 256;
        k_relu_mask_dy<<<(unsigned)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, s>>>(
            (const uint4*)dy, (const uint4*)y, (uint4*)dy_masked, n8);
        dsrc = dy_masked;
    }
    CUtensorMap t1, t2, td;
    if (!act_map(&t1, x1, c1, n, h, w, WG_PX) || !act_map(&td, dsrc, cout, n, h, w, WG_PX)) return 0;
    if (c2 > 0) {
        if (!act_map(&t2, x2, c2, n, h, w, WG_PX)) return 0;
    } else {
        t2 = t1;
    }
    static cudaError_t attr = cudaFuncSetAttribute(k_conv_wgrad_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, WG_SMEM);
    if (attr != cudaSuccess) return 0;
    int nz = 0, chunk = 0;
    glnn_tc_wgrad_plan(n, h, w, c1 + c2, cout, &nz, &chunk);
    dim3 grid((unsigned)(5 * ((c1 + c2) / 64) * (cout / 64)), (unsigned)nz);
    k_conv_wgrad_tma<<<grid, NTH, WG_SMEM, s>>>(t1, t2, td, ws, c1, c2, cout, h, w, (int)P, chunk, err);
    return 1;
}

static int conv_tc_args_ok(int c1, int c2, int n, int h, int w, int cout) {
    return n > 0 && h > 0 && w > 0 && c1 > 0 && c1 % 8 == 0 && c2 >= 0 && c2 % 8 == 0 && cout > 0 && cout % 8 == 0 &&
           (long long)n * h * w < (1LL << 31);
}

extern "C" {

int glnn_set_conv_tma(int32_t enable) {
    g_conv_tma = enable <= 0 ? 0 : (enable == 1 ? 1 : 2);
    return GLGPU_OK;
}

int glnn_conv3x3_fwd(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* wb, const float* bias,
                        void* y, int32_t n, int32_t h, int32_t w, int32_t cout, int32_t relu, int32_t* err,
                        void* stream) {
    if (!x1 || !wb || !bias || !y || !err || (c2 > 0 && !x2) || !conv_tc_args_ok(c1, c2, n, h, w, cout)) return GLGPU_E_ARG;
    if (((uintptr_t)x1 | (uintptr_t)x2 | (uintptr_t)wb | (uintptr_t)y) & 15u) return GLGPU_E_ARG;
    const long long P = (long long)n * h * w;
    dim3 grid((unsigned)((P + TM - 1) / TM), (unsigned)((cout + TN - 1) / TN));
    cudaStream_t s = (cudaStream_t)stream;
    if (conv_fwd_tma(x1, c1, x2, c2, wb, bias, y, n, h, w, cout, relu, err, s))
        return cudaGetLastError() == cudaSuccess ? GLGPU_OK : GLGPU_E_CUDA;
    if ((relu ? conv_tc_smem_attr<0, 1>() : conv_tc_smem_attr<0, 0>()) != cudaSuccess) return GLGPU_E_CUDA;
    if (relu)
        k_conv_tc<0, 1><<<grid, NTH, SMEM_BYTES, s>>>((const bf16*)x1, c1, (const bf16*)x2, c2, nullptr, (const bf16*)wb,
                                                     bias, (bf16*)y, cout, nullptr, 0, n, h, w, err);
    else
        k_conv_tc<0, 0><<<grid, NTH, SMEM_BYTES, s>>>((const bf16*)x1, c1, (const bf16*)x2, c2, nullptr, (const bf16*)wb,
                                                     bias, (bf16*)y, cout, nullptr, 0, n, h, w, err);
    return cudaGetLastError() == cudaSuccess ? GLGPU_OK : GLGPU_E_CUDA;
}

int glnn_relu_mask(const void* dy, const void* y, void* out, int64_t count, void* stream) {
    if (!dy || !y || !out || count < 0 || count % 8 != 0) return GLGPU_E_ARG;
    if (((uintptr_t)dy | (uintptr_t)y | (uintptr_t)out) & 15u) return GLGPU_E_ARG;
    const long long n8 = count / 8;
    if (n8 == 0) return GLGPU_OK;
    const long long blocks = (n8 + 255) / 256;
    k_relu_mask_dy<<<(unsigned)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, (cudaStream_t)stream>>>(
        (const uint4*)dy, (const uint4*)y, (uint4*)out, n8);
    return cudaGetLastError() == cudaSuccess ? GLGPU_OK : GLGPU_E_CUDA;
}

int glnn_conv3x3_bwd_data(const void* dy, const void* y, int32_t relu, const void* wt, void* dx1, int32_t c1,
                             void* dx2, int32_t c2, int32_t n, int32_t h, int32_t w, int32_t cout, int32_t* err,
                             void* stream) {
    if (!dy || !wt || !dx1 || !err || (relu && !y) || (c2 > 0 && !dx2) || !conv_tc_args_ok(c1, c2, n, h, w, cout))
        return GLGPU_E_ARG;
    if (((uintptr_t)dy | (uintptr_t)y | (uintptr_t)wt | (uintptr_t)dx1 | (uintptr_t)dx2) & 15u) return GLGPU_E_ARG;
    const long long P = (long long)n * h * w;
    dim3 grid((unsigned)((P + TM - 1) / TM), (unsigned)((c1 + c2 + TN - 1) / TN));
    cudaStream_t s = (cudaStream_t)stream;
    if (!relu && conv_bwd_data_tma(dy, wt, dx1, c1, dx2, c2, n, h, w, cout, err, s))
        return cudaGetLastError() == cudaSuccess ? GLGPU_OK : GLGPU_E_CUDA;
    if ((relu ? conv_tc_smem_attr<1, 1>() : conv_tc_smem_attr<1, 0>()) != cudaSuccess) return GLGPU_E_CUDA;
    if (relu)
        k_conv_tc<1, 1><<<grid, NTH, SMEM_BYTES, s>>>((const bf16*)dy, cout, nullptr, 0, (const bf16*)y, (const bf16*)wt,
                                                     nullptr, (bf16*)dx1, c1, (bf16*)dx2, c2, n, h, w, err);
    else
        k_conv_tc<1, 0><<<grid, NTH, SMEM_BYTES, s>>>((const bf16*)dy, cout, nullptr, 0, nullptr, (const bf16*)wt,
                                                     nullptr, (bf16*)dx1, c1, (bf16*)dx2, c2, n, h, w, err);
    return cudaGetLastError() == cudaSuccess ? GLGPU_OK : GLGPU_E_CUDA;
}

}  // extern "C"
