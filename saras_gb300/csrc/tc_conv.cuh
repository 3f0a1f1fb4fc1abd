// tc_conv.cuh -- 3x3x3 convolution as an implicit GEMM on the 5th-generation
// tensor cores (tcgen05), BF16 operands, FP32 accumulation in tensor memory.
//
// GEMM view (channels-last activations X[z][y][x][C]):
//   out[m][n] = sum_k A[m][k] * B[n][k],   m = output voxel, n = output channel,
//   k = (tap, input channel), 27 taps, input channels in chunks of 16.
// One CTA (4 warps) owns 128 consecutive output voxels (M = 128) and all N
// output channels.  Each K step is one tcgen05.mma (K = 16): the A tile (128
// voxels x 16 channels of one tap, gathered with cp.async, zero outside the
// domain) and the B tile (N x 16 packed weights) sit in shared memory in the
// canonical K-major layout without swizzle: 8x8 "core matrices" of 128 bytes,
// K-adjacent core matrices 128 B apart (leading byte offset), M/N-adjacent
// ones 256 B apart (stride byte offset).  A four-stage ring overlaps the
// gathers with the MMAs; tcgen05.commit arrives on a per-stage mbarrier that
// releases the stage for reuse.  The accumulator (128 lanes x N FP32 columns)
// is read back with tcgen05.ld: warp w reads lanes 32w..32w+31, i.e. thread t
// of the CTA reads the N channels of voxel t, matching channels-last storage.
//
// Every mbarrier wait is bounded; on timeout the kernel raises an error flag,
// drains its own cp.async groups, frees its tensor memory and returns.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

#include "tma.cuh"

namespace saras {

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(slot)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

__device__ __forceinline__ void tc_mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t *m) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(su32(m)) : "memory");
}
// 32 lanes x 16 consecutive 32-bit columns per warp.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// Shared-memory matrix descriptor: start address, leading / stride byte
// offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

struct ConvArgs {
    const __nv_bfloat16 *in0, *in1;   // channels-last inputs (concatenated along C)
    int c0, c1;                       // their channel counts (multiples of 16; c1 may be 0)
    const __nv_bfloat16 *wpk;         // packed weights, one N x 16 tile per K step
    const float *bias;                // N, or null
    __nv_bfloat16 *out0, *out1;       // BF16 outputs: channels [0, split) and [split, N)
    int split;
    float *out32;                     // FP32 output of channel 0 only (final layer), or null
    const __nv_bfloat16 *mask0, *mask1;  // zero the output where the mask is <= 0 (ReLU backward)
    int relu;
    int D, H, W;
    int nvox;
    int *err;
};

constexpr int kConvStages = 4;
constexpr int kConvTileBytesA = 128 * 16 * 2;

template <int N>
__host__ __device__ constexpr int conv_smem_bytes() { return kConvStages * (kConvTileBytesA + N * 32) + 128; }
template <int N>
__host__ __device__ constexpr uint32_t conv_tmem_cols() { return N <= 32 ? 32u : N <= 64 ? 64u : 128u; }

template <int N>
__global__ void __launch_bounds__(128) k_conv3d_tc(ConvArgs a) {
    static_assert(N % 16 == 0 && N >= 16 && N <= 128, "N");
    extern __shared__ __align__(128) uint8_t smem[];
    constexpr int SB = kConvTileBytesA + N * 32;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kConvStages * SB);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + kConvStages);
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t NCOLS = conv_tmem_cols<N>();
    constexpr uint32_t IDESC = idesc_bf16(128, N);

    if (warp == 0) { tmem_alloc(tslot, NCOLS); tmem_relinquish(); }
    if (tid == 0) {
        for (int s = 0; s < kConvStages; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tslot;

    // this thread's output voxel
    const int v = blockIdx.x * 128 + tid;
    const bool valid = v < a.nvox;
    int z = 0, y = 0, x = 0;
    if (valid) { x = v % a.W; int t = v / a.W; y = t % a.H; z = t / a.H; }
    const int nch0 = a.c0 >> 4, nch = (a.c0 + a.c1) >> 4;
    const int nsteps = 27 * nch;

    auto load_step = [&](int s, int st) {
        int tap = s / nch, ch = s - tap * nch;
        int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const __nv_bfloat16 *src;
        int cs, co;
        if (ch < nch0) { src = a.in0; cs = a.c0; co = ch << 4; }
        else { src = a.in1; cs = a.c1; co = (ch - nch0) << 4; }
        int zz = z + dz, yy = y + dy, xx = x + dx;
        bool ok = valid && zz >= 0 && zz < a.D && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
        long sv = ok ? ((long)(zz * a.H + yy) * a.W + xx) : 0;
        const __nv_bfloat16 *g = src + sv * cs + co;
        uint32_t dA = su32(smem + st * SB) + (tid >> 3) * 256 + (tid & 7) * 16;
        cp_async16(dA, g, ok ? 16 : 0);
        cp_async16(dA + 128, g + 8, ok ? 16 : 0);
        const uint8_t *wsrc = reinterpret_cast<const uint8_t *>(a.wpk) + (long)s * N * 32;
        uint32_t dB = su32(smem + st * SB + kConvTileBytesA);
        for (int q = tid; q < N * 2; q += 128) cp_async16(dB + q * 16, wsrc + q * 16, 16);
    };

    bool ok = true;
#pragma unroll 1
    for (int s = 0; s < kConvStages - 1; ++s) {
        if (s < nsteps) load_step(s, s);
        cp_async_commit();
    }
#pragma unroll 1
    for (int s = 0; s < nsteps; ++s) {
        const int st = s % kConvStages;
        cp_async_wait<kConvStages - 2>();
        __syncthreads();
        fence_async_smem();
        if (tid == 0 && ok) {
            tc_fence_after();
            uint32_t aAddr = su32(smem + st * SB), bAddr = aAddr + kConvTileBytesA;
            tc_mma_bf16(taddr, smem_desc(aAddr, 128, 256), smem_desc(bAddr, 128, 256), IDESC, s > 0 ? 1u : 0u);
            tc_commit(&mbar[st]);
        }
        const int ns = s + kConvStages - 1;
        if (ns < nsteps) {
            const int nst = ns % kConvStages;
            // stage nst was last read by the MMA of step ns - kConvStages (= s - 1)
            if (ns >= kConvStages && ok) ok = mbar_wait(&mbar[nst], (uint32_t)(((ns - kConvStages) / kConvStages) & 1), a.err);
            if (ok) load_step(ns, nst);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    // all MMAs done once the last commit has arrived
    if (ok) {
        const int last = nsteps - 1;
        ok = mbar_wait(&mbar[last % kConvStages], (uint32_t)((last / kConvStages) & 1), a.err);
    }
    __syncthreads();
    tc_fence_after();
    if (ok) {
        const uint32_t tw = taddr + ((uint32_t)(warp * 32) << 16);
        if (a.out32) {
            float vals[16];
            tc_ld16(tw, vals);
            if (valid) a.out32[v] = vals[0] + (a.bias ? a.bias[0] : 0.0f);
        } else {
#pragma unroll
            for (int q = 0; q < N / 16; ++q) {
                float vals[16];
                tc_ld16(tw + q * 16, vals);
                if (valid) {
                    __align__(16) __nv_bfloat16 o[16];
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        int n = q * 16 + e;
                        float t = vals[e] + (a.bias ? a.bias[n] : 0.0f);
                        if (a.relu) t = fmaxf(t, 0.0f);
                        o[e] = __float2bfloat16(t);
                    }
                    int n0 = q * 16;
                    __nv_bfloat16 *dst;
                    const __nv_bfloat16 *msk;
                    if (n0 < a.split) { dst = a.out0 + (long)v * a.split + n0; msk = a.mask0 ? a.mask0 + (long)v * a.split + n0 : nullptr; }
                    else { dst = a.out1 + (long)v * (N - a.split) + (n0 - a.split); msk = a.mask1 ? a.mask1 + (long)v * (N - a.split) + (n0 - a.split) : nullptr; }
                    if (msk) {
#pragma unroll
                        for (int e = 0; e < 16; ++e)
                            if (!(__bfloat162float(msk[e]) > 0.0f)) o[e] = __float2bfloat16(0.0f);
                    }
                    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
                    const uint4 *s4 = reinterpret_cast<const uint4 *>(o);
                    d4[0] = s4[0];
                    d4[1] = s4[1];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(taddr, NCOLS);
}

// ---- weight gradient on the tensor cores
// dW[n][tap][c] = sum_v dY[v][n] X[v + off(tap)][c] as the GEMM
//   D[m][n] = sum_k A[m][k] B[n][k],  m = tap * Cin + c (27 Cin rows in tiles
//   of 128), n = output channel, k = voxel.
// Both operands are staged MN-major, which is the order the channels-last
// tensors already have: one 16-byte row of a core matrix is 8 consecutive
// channels of one voxel (X at the shifted voxel for A, dY for B), so every row
// is one 16-byte cp.async straight from global memory.  Core matrices adjacent
// along M (or N) are 128 B apart (the stride byte offset of a no-swizzle
// MN-major descriptor), the two 8-voxel halves of a K step of 16 voxels
// 16 x 128 B (A) or N / 8 x 128 B (B) apart (its leading byte offset; a first
// build with the two exchanged read past the tile, into the reserve below, and
// produced wrong sums, not a fault).  Each CTA reduces a chunk of voxels for one M tile
// into its tensor-memory accumulator and adds it to the FP32 dW with atomics;
// the CTAs of M tile 0 also add their chunk's sum of dY to db.
struct DwArgs {
    const __nv_bfloat16 *in0, *in1;   // X, channels-last, concatenated along C
    int c0, c1;
    const __nv_bfloat16 *dy;          // dY, channels-last, N channels
    float *dw;                        // [N][27][c0 + c1]
    float *db;                        // [N], or null
    int D, H, W, nvox;
    int chunk;                        // voxels a CTA reduces (a multiple of 16)
    int *err;
};

constexpr int kDwStages = 4;
constexpr int kDwTileA = 128 * 16 * 2;
// Reserve: the ring is followed by 32 KB that no operand occupies, so that even
// a descriptor read with its two byte offsets exchanged (15 x 2048 B past a
// stage at most) stays inside the CTA's shared memory.
constexpr int kDwReserve = 32768;
template <int N>
__host__ __device__ constexpr int dw_stage_bytes() { return kDwTileA + N * 32; }
template <int N>
__host__ __device__ constexpr int dw_smem_bytes() { return kDwStages * dw_stage_bytes<N>() + kDwReserve + 128; }

template <int N>
__global__ void __launch_bounds__(128) k_conv_dw_tc(DwArgs a) {
    static_assert(N % 16 == 0 && N >= 16 && N <= 128, "N");
    extern __shared__ __align__(128) uint8_t smem[];
    constexpr int SB = dw_stage_bytes<N>();
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + kDwStages * SB + kDwReserve);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + kDwStages);
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t NCOLS = conv_tmem_cols<N>();
    constexpr uint32_t IDESC = idesc_bf16(128, N) | (1u << 15) | (1u << 16);   // A and B MN-major
    const int cin = a.c0 + a.c1, mtot = 27 * cin;
    const int mt = blockIdx.y;
    const long v0 = (long)blockIdx.x * a.chunk;
    const long v1 = min(v0 + (long)a.chunk, (long)a.nvox);
    const int nsteps = v1 > v0 ? (int)((v1 - v0 + 15) / 16) : 0;

    if (warp == 0) { tmem_alloc(tslot, NCOLS); tmem_relinquish(); }
    if (tid == 0) {
        for (int s = 0; s < kDwStages; ++s) mbar_init(&mbar[s], 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tslot;

    auto load_step = [&](int s, int st) {
        const uint32_t base = su32(smem + st * SB);
        const long vb = v0 + (long)s * 16;
#pragma unroll
        for (int h = 0; h < 2; ++h) {   // A: 16 M groups x 16 voxel rows, two rows a thread
            const int cidx = tid + h * 128, mg = cidx >> 4, r = cidx & 15;
            const int m0 = mt * 128 + mg * 8;
            const long v = vb + r;
            const __nv_bfloat16 *src = a.in0;
            bool ok = m0 < mtot && v < v1;
            if (ok) {
                const int tap = m0 / cin, c = m0 - tap * cin;
                const int x = (int)(v % a.W);
                const long t = v / a.W;
                const int y = (int)(t % a.H), z = (int)(t / a.H);
                const int zz = z + tap / 9 - 1, yy = y + (tap / 3) % 3 - 1, xx = x + tap % 3 - 1;
                ok = zz >= 0 && zz < a.D && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
                if (ok) {
                    const long sv = ((long)zz * a.H + yy) * a.W + xx;
                    src = c < a.c0 ? a.in0 + sv * a.c0 + c : a.in1 + sv * a.c1 + (c - a.c0);
                }
            }
            cp_async16(base + mg * 128 + (r & 7) * 16 + (r >> 3) * 2048, src, ok ? 16 : 0);
        }
        for (int cidx = tid; cidx < N * 2; cidx += 128) {   // B: N / 8 groups x 16 voxel rows
            const int ng = cidx >> 4, r = cidx & 15;
            const long v = vb + r;
            const bool ok = v < v1;
            cp_async16(base + kDwTileA + ng * 128 + (r & 7) * 16 + (r >> 3) * (N / 8) * 128, ok ? a.dy + v * N + ng * 8 : a.dy,
                       ok ? 16 : 0);
        }
    };

    bool ok = true;
#pragma unroll 1
    for (int s = 0; s < kDwStages - 1; ++s) {
        if (s < nsteps) load_step(s, s);
        cp_async_commit();
    }
#pragma unroll 1
    for (int s = 0; s < nsteps; ++s) {
        const int st = s % kDwStages;
        cp_async_wait<kDwStages - 2>();
        __syncthreads();
        fence_async_smem();
        if (tid == 0 && ok) {
            tc_fence_after();
            const uint32_t aAddr = su32(smem + st * SB), bAddr = aAddr + kDwTileA;
            // no-swizzle MN-major: the stride byte offset steps between core
            // matrices along M / N, the leading byte offset along K
            tc_mma_bf16(taddr, smem_desc(aAddr, 2048, 128), smem_desc(bAddr, (N / 8) * 128, 128), IDESC, s > 0 ? 1u : 0u);
            tc_commit(&mbar[st]);
        }
        const int ns = s + kDwStages - 1;
        if (ns < nsteps) {
            const int nst = ns % kDwStages;
            // stage nst was last read by the MMA of step ns - kDwStages (= s - 1)
            if (ns >= kDwStages && ok) ok = mbar_wait(&mbar[nst], (uint32_t)(((ns - kDwStages) / kDwStages) & 1), a.err);
            if (ok) load_step(ns, nst);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    if (ok && nsteps > 0) {
        const int last = nsteps - 1;
        ok = mbar_wait(&mbar[last % kDwStages], (uint32_t)((last / kDwStages) & 1), a.err);
    }
    __syncthreads();
    tc_fence_after();
    if (ok && nsteps > 0) {
        const int m = mt * 128 + tid;
        const int tap = m / cin, c = m - tap * cin;
        const uint32_t tw = taddr + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int q = 0; q < N / 16; ++q) {
            float vals[16];
            tc_ld16(tw + q * 16, vals);
            if (m < mtot) {
#pragma unroll
                for (int e = 0; e < 16; ++e) atomicAdd(&a.dw[((long)(q * 16 + e) * 27 + tap) * cin + c], vals[e]);
            }
        }
    }
    if (a.db && mt == 0 && tid < N) {
        float sum = 0.0f;
        for (long v = v0; v < v1; ++v) sum += __bfloat162float(a.dy[v * N + tid]);
        atomicAdd(&a.db[tid], sum);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(taddr, NCOLS);
}

}  // namespace saras
