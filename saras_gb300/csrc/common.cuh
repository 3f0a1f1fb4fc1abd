// common.cuh -- shared device/host definitions of the GB300 SARAS library.
//
// Layout: every field is a padded box in the reference layout (C order, k
// fastest, ghost width 1, logical indices -1..n per axis), so host arrays of
// the reference copy in and out with one memcpy.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/saras_gb300.h"

namespace saras {

// ------------------------------------------------------------------ views
template <typename T>
struct View3 {
    T *p = nullptr;
    int n[3] = {0, 0, 0};     // core counts; logical index range -1..n[d]
    long sx = 0, sy = 0;      // strides of i and j (k stride is 1)
    __host__ __device__ inline long off(int i, int j, int k) const {
        return (long)(i + 1) * sx + (long)(j + 1) * sy + (k + 1);
    }
    __host__ __device__ inline T &operator()(int i, int j, int k) const { return p[off(i, j, k)]; }
    __host__ __device__ inline long size() const { return (long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2); }
};

template <typename T>
inline View3<T> make_view(T *p, int nx, int ny, int nz) {
    View3<T> v;
    v.p = p; v.n[0] = nx; v.n[1] = ny; v.n[2] = nz;
    v.sy = nz + 2; v.sx = (long)(ny + 2) * (nz + 2);
    return v;
}

// ------------------------------------------------------------------ boundary programs
// A field boundary fill (syncData followed by the wall objects, in the order
// hydro::imposeUBCs applies them) is a short list of plane operations.  Each
// op writes a box of ghost/wall points; its value is a constant, a copy of the
// point displaced by `shift`, or 2c - (that copy).  The device resolves the
// final value of any point by walking the list backwards (see bc_resolve).
enum BcOpKind : int { OP_CONST = 0, OP_COPY = 1, OP_REFLECT = 2 };
struct BcOp {
    int kind;
    int lo[3], hi[3];   // target box (inclusive)
    int shift[3];       // source = target + shift
    double c;
};
constexpr int kMaxBcOps = 16;
struct BcProgram {
    int nops = 0;
    BcOp op[kMaxBcOps];
    int blo[3], bhi[3];  // bulk box (points never targeted by an op)
};

// Resolve the value that the program leaves at (i,j,k), given base(q) = value
// of point q before the program ran.  Chains are at most nops long; the op
// values are replayed forward in program order so the arithmetic matches the
// sequential plane operations exactly.
template <typename BaseFn>
__device__ __forceinline__ double bc_resolve(const BcProgram &prog, int i, int j, int k, BaseFn base) {
    int chain[kMaxBcOps];
    int nchain = 0;
    double value = 0.0;
    bool haveConst = false;
    int q[3] = {i, j, k};
    for (int o = prog.nops - 1; o >= 0; --o) {
        const BcOp &op = prog.op[o];
        if (q[0] < op.lo[0] || q[0] > op.hi[0] || q[1] < op.lo[1] || q[1] > op.hi[1] || q[2] < op.lo[2] || q[2] > op.hi[2])
            continue;
        if (op.kind == OP_CONST) { value = op.c; haveConst = true; break; }
        chain[nchain++] = o;
        q[0] += op.shift[0]; q[1] += op.shift[1]; q[2] += op.shift[2];
    }
    if (!haveConst) value = base(q[0], q[1], q[2]);
    for (int c = nchain - 1; c >= 0; --c) {
        const BcOp &op = prog.op[chain[c]];
        if (op.kind == OP_REFLECT) value = 2.0 * op.c - value;
    }
    return value;
}

__host__ __device__ inline bool in_box(const int lo[3], const int hi[3], int i, int j, int k) {
    return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
}

// ------------------------------------------------------------------ reductions
// Non-negative doubles order like their bit patterns, so atomicMax on the
// 64-bit pattern is an exact max.
__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide max of non-negative values into *out (atomic), exact, on the
// 64-bit patterns (integer pipe; NaN stays above Inf).
__device__ __forceinline__ void block_max_bits_to(unsigned long long u, double *out) {
    __shared__ unsigned long long sm[32];
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long x = __shfl_xor_sync(0xffffffffu, u, o);
        u = x > u ? x : u;
    }
    int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    int lane = tid & 31, w = tid >> 5;
    __syncthreads();
    if (lane == 0) sm[w] = u;
    __syncthreads();
    if (w == 0) {
        unsigned long long x = lane < nw ? sm[lane] : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
            x = y > x ? y : x;
        }
        if (lane == 0 && x > 0ull) atomicMax(reinterpret_cast<unsigned long long *>(out), x);
    }
}

// |v| as the integer that orders like it (for running maxima off the FP64 pipe).
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

__device__ __forceinline__ void block_max_to(double v, double *out) { block_max_bits_to(abs_bits(v), out); }

// Block-wide max of |v| for float values into the double *out (atomic), on
// the integer bits: non-negative floats order like their bit patterns, NaN
// above Inf, so a NaN anywhere reaches *out as NaN.  redux.sync does the warp
// step in one instruction; a warp max in FP64 would cost GB300's FP64 pipe
// about as much as a stencil.
__device__ __forceinline__ void block_maxf_to(float v, double *out) {
    __shared__ unsigned smf[32];
    unsigned u = __reduce_max_sync(0xffffffffu, __float_as_uint(v) & 0x7fffffffu);
    int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    int lane = tid & 31, w = tid >> 5;
    __syncthreads();
    if (lane == 0) smf[w] = u;
    __syncthreads();
    if (w == 0) {
        unsigned x = lane < nw ? smf[lane] : 0u;
        x = __reduce_max_sync(0xffffffffu, x);
        if (lane == 0 && x > 0u) atomic_max_nonneg(out, (double)__uint_as_float(x));
    }
}

// ------------------------------------------------------------------ errors
#define SARAS_CUDA_TRY(expr)                                                          \
    do {                                                                              \
        cudaError_t _e = (expr);                                                      \
        if (_e != cudaSuccess) {                                                      \
            ::saras::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));  \
            return SARAS_CUDA_ERROR;                                                  \
        }                                                                             \
    } while (0)

void set_error(const std::string &msg);

}  // namespace saras
