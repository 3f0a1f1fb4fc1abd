// unet.cu -- learned warm start for the pressure-correction solve.
//
// A three-level 3D U-Net (16/32/64 channels, 3x3x3 convolutions, BF16
// activations and weights, FP32 accumulation on tcgen05 tensor cores) maps
//   (b / s_b, P_{n-1} / s_p, P_{n-2} / s_p)   at multigrid level 1
// to a correction d of the linear extrapolation 2 P_{n-1} - P_{n-2}; the guess
// handed to the multigrid solve is
//   P_guess = 2 P_{n-1} - P_{n-2} + s_p * prolong(d),
// and the solver keeps the previous pressure instead whenever the guess has the
// larger FP64 residual.  The network is trained on (input, solution) pairs that
// the solver itself produces during the run's warm-up, with Adam on FP32
// master weights; forward and input-gradient convolutions (k_conv3d_tc) and
// the weight gradients (k_conv_dw_tc, a GEMM whose K runs over voxels) all run
// on the tensor cores.

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>
#include <type_traits>

#include "context.cuh"
#include "tc_conv.cuh"
#include "df64.cuh"

namespace saras {

__global__ void k_final_reduce(const double *part, int n, int op, double *out);
typedef __nv_bfloat16 bf16;

// ------------------------------------------------------------------ element kernels
struct Grid3 {
    int D, H, W;
    __host__ __device__ long n() const { return (long)D * H * W; }
};

__device__ __forceinline__ float fw1(int d) { return d == 0 ? 0.5f : 0.25f; }

// Full-weighting restriction of a channels-last tensor (vertex grids, coarse
// point i sits on fine point 2i; zero outside the fine grid), times `scale`.
__global__ void k_pool_down(const bf16 *__restrict__ in, bf16 *__restrict__ out, int C, Grid3 f, Grid3 c, float scale) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long total = c.n() * C;
    if (t >= total) return;
    int ch = (int)(t % C);
    long v = t / C;
    int x = (int)(v % c.W), y = (int)((v / c.W) % c.H), z = (int)(v / ((long)c.W * c.H));
    float s = 0.0f;
    for (int dz = -1; dz <= 1; ++dz) {
        int zz = 2 * z + dz;
        if (zz < 0 || zz >= f.D) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = 2 * y + dy;
            if (yy < 0 || yy >= f.H) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = 2 * x + dx;
                if (xx < 0 || xx >= f.W) continue;
                s += fw1(dz) * fw1(dy) * fw1(dx) * __bfloat162float(in[(((long)zz * f.H + yy) * f.W + xx) * C + ch]);
            }
        }
    }
    out[t] = __float2bfloat16(s * scale);
}

// Trilinear vertex prolongation of a channels-last tensor, times `scale`.
__global__ void k_pool_up(const bf16 *__restrict__ in, bf16 *__restrict__ out, int C, Grid3 c, Grid3 f, float scale) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long total = f.n() * C;
    if (t >= total) return;
    int ch = (int)(t % C);
    long v = t / C;
    int x = (int)(v % f.W), y = (int)((v / f.W) % f.H), z = (int)(v / ((long)f.W * f.H));
    int x0 = x >> 1, y0 = y >> 1, z0 = z >> 1;
    int x1 = min(x0 + (x & 1), c.W - 1), y1 = min(y0 + (y & 1), c.H - 1), z1 = min(z0 + (z & 1), c.D - 1);
    auto at = [&](int a, int b, int d) { return __bfloat162float(in[(((long)a * c.H + b) * c.W + d) * C + ch]); };
    float s = at(z0, y0, x0) + at(z0, y0, x1) + at(z0, y1, x0) + at(z0, y1, x1) + at(z1, y0, x0) + at(z1, y0, x1) +
              at(z1, y1, x0) + at(z1, y1, x1);
    out[t] = __float2bfloat16(0.125f * s * scale);
}

// out = (a + b) where mask > 0, else 0  (b and mask optional).
__global__ void k_add_mask(const bf16 *a, const bf16 *b, const bf16 *mask, bf16 *out, long n) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    float v = __bfloat162float(a[t]) + (b ? __bfloat162float(b[t]) : 0.0f);
    if (mask && !(__bfloat162float(mask[t]) > 0.0f)) v = 0.0f;
    out[t] = __float2bfloat16(v);
}

// Pack FP32 master weights W[cout][27][cin] into the per-K-step tensor-core
// tiles of k_conv3d_tc.  transposed = 0: forward tiles (N = cout, K = cin);
// transposed = 1: input-gradient tiles (N = cin, K = cout, taps mirrored).
__global__ void k_pack_weights(const float *__restrict__ w, bf16 *__restrict__ pk, int cin, int cout, int transposed) {
    int N = transposed ? cin : cout, KC = transposed ? cout : cin;
    int nch = KC / 16;
    long total = 27L * nch * N * 16;
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= total) return;
    int k = (int)(t % 16);
    int n = (int)((t / 16) % N);
    long s = t / (16L * N);
    int tap = (int)(s / nch), ch = (int)(s % nch);
    int kk = ch * 16 + k;
    float val = transposed ? w[((long)kk * 27 + (26 - tap)) * cin + n] : w[((long)n * 27 + tap) * cin + kk];
    long byte = s * (long)N * 32 + (n >> 3) * 256 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2;
    pk[byte / 2] = __float2bfloat16(val);
}

// Adam on the flat FP32 parameter vector.
__global__ void k_adam(float *p, const float *g, float *m, float *v, long n, float lr, float b1, float b2, float eps, float c1, float c2) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    float gr = g[t];
    float mm = b1 * m[t] + (1.0f - b1) * gr;
    float vv = b2 * v[t] + (1.0f - b2) * gr * gr;
    m[t] = mm;
    v[t] = vv;
    p[t] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// ---- FP64 <-> network features
// The network works on multigrid level lb (the first level with at most 65
// points per axis, so its cost does not grow with the grid), fed by full-
// weighting restrictions of the divergence b and of the pressure history.
struct L0View {
    const double *p;
    int n[3];     // core upper index (E) per axis; padded extent E+3
    __device__ double at(int i, int j, int k) const {
        return p[((long)(i + 1) * (n[1] + 3) + (j + 1)) * (n[2] + 3) + (k + 1)];
    }
};

// Level-0 padded field -> level-1 core array: full weighting (coarse point i on
// fine point 2i, weights (1/64) [1 2 1]^3, taps outside the grid skipped).  In
// FP64 the 27 fused multiply-adds a coarse point are bound by GB300's FP64
// pipe; here every fine value is split into a float pair (integer work) and
// the separable sums run in float-pair arithmetic (about 2^-44 of the largest
// tap), one FP64 addition a coarse point.  One thread per coarse (y, x)
// column marches kR0Ch coarse planes, the odd fine plane between two coarse
// planes serving both.
constexpr int kR0Ch = 8;

__global__ void __launch_bounds__(256) k_restrict0(L0View f, Grid3 g1, double *out) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z0 = blockIdx.z * kR0Ch;
    if (x >= g1.W || y >= g1.H) return;
    const int zend = min(z0 + kR0Ch, g1.D);
    auto plane = [&](int zz) -> fpair {   // in-plane [1 2 1] x [1 2 1] sum of fine plane zz (0 outside)
        fpair s = fpair{0.0f, 0.0f};
        if (zz < 0 || zz > f.n[0]) return s;
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = 2 * y + dy;
            if (yy < 0 || yy > f.n[1]) continue;
            fpair r = fpair{0.0f, 0.0f};
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = 2 * x + dx;
                if (xx < 0 || xx > f.n[2]) continue;
                fpair v = fp_of(f.at(zz, yy, xx));
                r = fp_add(r, dx == 0 ? fpair{2.0f * v.h, 2.0f * v.l} : v);
            }
            s = fp_add(s, dy == 0 ? fpair{2.0f * r.h, 2.0f * r.l} : r);
        }
        return s;
    };
    fpair lo = plane(2 * z0 - 1);
    for (int z = z0; z < zend; ++z) {
        fpair mid = plane(2 * z), hi = plane(2 * z + 1);
        fpair t = fp_add(fp_add(lo, fpair{2.0f * mid.h, 2.0f * mid.l}), hi);
        out[((long)z * g1.H + y) * g1.W + x] = (f2d(t.h) + f2d(t.l)) * 0.015625;
        lo = hi;
    }
}

// Level-l core array -> level-l+1 core array, the same weights (FP64; these
// levels are small).
__global__ void k_restrict(const double *f, Grid3 gf, Grid3 gc, double *out) {
    long v = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (v >= gc.n()) return;
    int x = (int)(v % gc.W), y = (int)((v / gc.W) % gc.H), z = (int)(v / ((long)gc.W * gc.H));
    double s = 0.0;
    for (int dz = -1; dz <= 1; ++dz) {
        int zz = 2 * z + dz;
        if (zz < 0 || zz >= gf.D) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = 2 * y + dy;
            if (yy < 0 || yy >= gf.H) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = 2 * x + dx;
                if (xx < 0 || xx >= gf.W) continue;
                s = fma((double)(fw1(dz) * fw1(dy) * fw1(dx)), f[((long)zz * gf.H + yy) * gf.W + xx], s);
            }
        }
    }
    out[v] = s;
}

// Scales of the features at level lb: s_b = max|R b|, s_d = max|R(P1 - P2)|,
// s_r = max|R r_ex| with R r_ex = R b - 2 R b1 + R b2 (the residual of the
// extrapolation 2 P1 - P2 is b - 2 b1 + b2 up to the previous solves'
// residuals, which the target keeps below 1e-8 of max|b|).
__global__ void k_feat_scales(const double *rb0, const double *rb1, const double *rb2, const double *rp0, const double *rp1, long n,
                              double *scales) {
    unsigned long long mb = 0, md = 0, mr = 0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        unsigned long long a = abs_bits(rb0[t]), d = abs_bits(rp0[t] - rp1[t]), r = abs_bits(rb0[t] - 2.0 * rb1[t] + rb2[t]);
        mb = a > mb ? a : mb;
        md = d > md ? d : md;
        mr = r > mr ? r : mr;
    }
    block_max_bits_to(mb, scales);
    block_max_bits_to(md, scales + 1);
    block_max_bits_to(mr, scales + 2);
}

// Network input (3 FP32 channels per level-lb point) and, with `target`, the
// training target d* = R(P_new - (2 P1 - P2)) / s_t:
//   0: R r_ex / s_r   1: R(P1 - P2) / s_d   2: R b / s_b
// with s_t = s_r L^2 / (4 pi^2) (the size A^-1 gives a residual of size s_r
// made of the domain's lowest modes).  scales = {s_b, s_d, s_r, -, -, s_t}.
__global__ void k_features(const double *rb0, const double *rb1, const double *rb2, const double *rp0, const double *rp1,
                           const double *rpnew, long n, const double *scales, float *feat, float *target) {
    long v = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (v >= n) return;
    feat[v * 3 + 0] = (float)((rb0[v] - 2.0 * rb1[v] + rb2[v]) / scales[2]);
    feat[v * 3 + 1] = (float)((rp0[v] - rp1[v]) / scales[1]);
    feat[v * 3 + 2] = (float)(rb0[v] / scales[0]);
    if (target) target[v] = (float)((rpnew[v] - (2.0 * rp0[v] - rp1[v])) / scales[5]);
}

// Expand 3-channel FP32 features into the 16-channel BF16 network input.
__global__ void k_expand(const float *feat, bf16 *x0, long nv) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= nv * 16) return;
    long v = t / 16;
    int c = (int)(t % 16);
    x0[t] = __float2bfloat16(c < 3 ? feat[v * 3 + c] : 0.0f);
}

// Loss 0.5 * mean (d - d*)^2 and the output gradient (channel 0 of a 16-channel BF16 tensor).
__global__ void k_loss(const float *d, const float *dstar, bf16 *gout, long nv, double *part) {
    __shared__ double sm[32];
    long v = blockIdx.x * (long)blockDim.x + threadIdx.x;
    double e = 0.0;
    if (v < nv) {
        float r = d[v] - dstar[v];
        e = 0.5 * (double)r * r;
        float gr = r / (float)nv;
#pragma unroll
        for (int c = 0; c < 16; ++c) gout[v * 16 + c] = __float2bfloat16(c == 0 ? gr : 0.0f);
    }
    e = warp_sum(e);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sm[w];
        part[blockIdx.x] = s;
    }
}

// Guess on level 0: 2 P1 - P2 (kind 1: 3 P1 - 3 P2 + P3, kind 2: P1 + P2 - P3) plus, with d, the
// network correction alpha s_t P(d), P the trilinear interpolation from level
// lb (repeated linear prolongation of vertex grids), at core points with the
// face-ghost images.  OT = long long: the guess goes straight into the
// fixed-point iterate, round(v 2^s) (flag set when out of range).
template <typename OT>
__global__ void k_apply_guess(OT *out, L0View p1, L0View p2, L0View p3, int kind, const float *d, Grid3 g, int lb,
                              const double *scales, const double *alpha, int per0, int per1, int per2, int s, int *flag) {
    // one thread per point of plane blockIdx.z, numbered k fastest over the
    // whole (j, k) plane (rows of 2^m + 1 points leave no idle warps)
    const int W = p1.n[2] + 1, t = blockIdx.x * blockDim.x + threadIdx.x, j = t / W, k = t - j * W, i = blockIdx.z;
    if (j > p1.n[1]) return;
    double v = kind == 1 ? 3.0 * (p1.at(i, j, k) - p2.at(i, j, k)) + p3.at(i, j, k)
             : kind == 2 ? (p1.at(i, j, k) + p2.at(i, j, k)) - p3.at(i, j, k)
                         : fma(2.0, p1.at(i, j, k), -p2.at(i, j, k));   // 2 P1 is exact: one rounding, as before
    if (d) {
        int m = (1 << lb) - 1;
        float inv = 1.0f / (float)(1 << lb);
        int z0 = i >> lb, y0 = j >> lb, x0 = k >> lb;
        float fz = (float)(i & m) * inv, fy = (float)(j & m) * inv, fx = (float)(k & m) * inv;
        int z1 = min(z0 + 1, g.D - 1), y1 = min(y0 + 1, g.H - 1), x1 = min(x0 + 1, g.W - 1);
        auto at = [&](int a, int b, int c) { return d[((long)a * g.H + b) * g.W + c]; };
        float c00 = at(z0, y0, x0) + fx * (at(z0, y0, x1) - at(z0, y0, x0));
        float c01 = at(z0, y1, x0) + fx * (at(z0, y1, x1) - at(z0, y1, x0));
        float c10 = at(z1, y0, x0) + fx * (at(z1, y0, x1) - at(z1, y0, x0));
        float c11 = at(z1, y1, x0) + fx * (at(z1, y1, x1) - at(z1, y1, x0));
        float c0 = c00 + fy * (c01 - c00), c1 = c10 + fy * (c11 - c10);
        v += (*alpha * scales[5]) * (double)(c0 + fz * (c1 - c0));
    }
    long sy = p1.n[2] + 3, sx = (long)(p1.n[1] + 3) * sy;
    OT w;
    if constexpr (std::is_same<OT, long long>::value) {
        bool bad = false;
        w = d2fx(v, s, bad);
        if (bad) atomicExch(flag, 1);
    } else {
        w = v;
    }
    auto put = [&](int a, int b, int c) { out[(long)(a + 1) * sx + (long)(b + 1) * sy + (c + 1)] = w; };
    put(i, j, k);
    int q[3] = {i, j, k};
    int per[3] = {per0, per1, per2};
    for (int dd = 0; dd < 3; ++dd) {
        int E = p1.n[dd];
        int g0 = -2, g1v = -2;
        if (per[dd]) { if (q[dd] == E - 1) g0 = -1; if (q[dd] == 1) g1v = E + 1; }
        else { if (q[dd] == 1) g0 = -1; if (q[dd] == E - 1) g1v = E + 1; }
        int r[3] = {i, j, k};
        if (g0 != -2) { r[dd] = g0; put(r[0], r[1], r[2]); }
        if (g1v != -2) { r[dd] = g1v; put(r[0], r[1], r[2]); }
    }
}

// Binomial low-pass filter ([1,2,1]/4 per axis, weights renormalised at the
// domain edge) of the network output: multigrid removes high-frequency error
// by itself, and BF16 rounding noise in the correction would otherwise show up
// amplified by the Laplacian in the residual of the guess.
__global__ void k_lowpass(const float *in, float *out, Grid3 g) {
    long v = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (v >= g.n()) return;
    int x = (int)(v % g.W), y = (int)((v / g.W) % g.H), z = (int)(v / ((long)g.W * g.H));
    float s = 0.0f, w = 0.0f;
    for (int dz = -1; dz <= 1; ++dz) {
        int zz = z + dz;
        if (zz < 0 || zz >= g.D) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = y + dy;
            if (yy < 0 || yy >= g.H) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = x + dx;
                if (xx < 0 || xx >= g.W) continue;
                float wt = fw1(dz) * fw1(dy) * fw1(dx);
                s += wt * in[((long)zz * g.H + yy) * g.W + xx];
                w += wt;
            }
        }
    }
    out[v] = s / w;
}

__global__ void k_floor_scale(double *s, double floor_, double lfac) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        for (int q = 0; q < 3; ++q)
            if (!(s[q] > floor_)) s[q] = floor_;
        s[5] = s[2] * lfac;
    }
}

constexpr int kAlphaBlocks = 152;   // one block per SM for the step-length reduction

// Step length of the network correction c = s_t d at level lb: with the
// restricted residual of the extrapolation R r_ex and q = A_lb c (the level's
// 7-point operator; mirror or periodic neighbours at the walls),
// alpha = <R r_ex, q> / <q, q> minimises |R r_ex - alpha q|_2, the residual the
// corrected guess leaves on the smooth modes the correction can change.
// per0 / l0 belong to the slowest axis (D, the reference's x), per2 / l2 to the fastest (W).
__global__ void k_alpha_coarse(const float *d, const double *rb0, const double *rb1, const double *rb2, Grid3 g, int per0, int per1,
                               int per2, double l0, double l1, double l2, const double *scales, double *part) {
    __shared__ double sm[2][32];
    double rq = 0.0, qq = 0.0;
    double st = scales[5];
    auto nb = [](int q, int E, int per, int dir) {   // neighbour index along one axis (E = last index)
        int r = q + dir;
        if (r < 0) r = per ? E - 1 : 1;
        if (r > E) r = per ? 1 : E - 1;
        return r;
    };
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < g.n(); t += (long)gridDim.x * blockDim.x) {
        int x = (int)(t % g.W), y = (int)((t / g.W) % g.H), z = (int)(t / ((long)g.W * g.H));
        auto at = [&](int a, int b, int c) { return (double)d[((long)a * g.H + b) * g.W + c]; };
        double C = at(z, y, x);
        double lap = l0 * (at(nb(z, g.D - 1, per0, 1), y, x) + at(nb(z, g.D - 1, per0, -1), y, x) - 2.0 * C) +
                     l1 * (at(z, nb(y, g.H - 1, per1, 1), x) + at(z, nb(y, g.H - 1, per1, -1), x) - 2.0 * C) +
                     l2 * (at(z, y, nb(x, g.W - 1, per2, 1)) + at(z, y, nb(x, g.W - 1, per2, -1)) - 2.0 * C);
        double q = st * lap;
        double re = rb0[t] - 2.0 * rb1[t] + rb2[t];
        rq += re * q;
        qq += q * q;
    }
    rq = warp_sum(rq);
    qq = warp_sum(qq);
    if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = rq; sm[1][threadIdx.x >> 5] = qq; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += sm[0][w]; c += sm[1][w]; }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = c;
    }
}

// alpha from the partial sums (fixed order), limited to [0, 1.5]; 0 when the
// correction has no effect on the residual or the sums are not finite.
__global__ void k_alpha_final(const double *part, int nb, double *alpha) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, c = 0.0;
    for (int q = 0; q < nb; ++q) { a += part[2 * q]; c += part[2 * q + 1]; }
    double al = (c > 0.0 && isfinite(a) && isfinite(c)) ? a / c : 0.0;
    *alpha = fmin(fmax(al, 0.0), 1.5);
}

// ------------------------------------------------------------------ host: network
struct ConvLayer {
    int cin0, cin1, cout, level;
    bool relu;
    long woff, boff;   // offsets of W and b in the flat parameter vector
    bf16 *wf = nullptr, *wt = nullptr;   // packed forward / transposed tiles
};

struct UNet {
    int lb = 1;                      // multigrid level of the network's finest grid
    Grid3 g[3];                      // levels lb, lb + 1, lb + 2
    std::vector<ConvLayer> L;
    long nparam = 0;
    float *param = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    long adam_t = 0;
    std::vector<bf16 *> act;          // activations
    std::vector<bf16 *> grd;          // gradient buffers
    bf16 *x0 = nullptr;
    float *out = nullptr, *feat = nullptr;
    double *scales = nullptr;         // s_b, s_d, s_r, last loss, step length alpha (device)
    // restrictions to level lb: b of this and the two previous solves, Pp of
    // the three previous solves (newest first), R(P_new) for training targets
    double *rb[3] = {nullptr, nullptr, nullptr}, *rp[3] = {nullptr, nullptr, nullptr}, *rpnew = nullptr;
    double *tmp[2] = {nullptr, nullptr};     // intermediate levels 1 .. lb-1 of a restriction
    int nb = 0, np = 0;                      // consecutive solves with rb / rp pushed
    bool bPushed = false;                    // rb[0] holds this solve's b
    bool track = false;                      // this solve pushes rb / rp
    bool wantNet = false;                    // the network was picked before its rings were complete
    bool shadow = false;                     // this solve builds both guesses
    // V-cycles per solve with the network's guess and with plain extrapolation
    // (moving averages), the basis of the choice between them
    double lrNet = 0.0, lrExt = 0.0;         // log10 of the start's residual / max|b|
    int usesNet = 0, usesExt = 0, solves = 0;
    int probeEvery = 8, nextProbe = 0;       // probe schedule of the guess that is not preferred
    bool preferNet = false;
    // training samples: 3 feature channels + target per voxel
    std::vector<float *> samples;
    int nsamples = 0, cap = 0, next = 0;
    int *err = nullptr;
    double *part = nullptr;
    bool trained = false;
    long flops_fwd = 0;
};

static int ucheck(Ctx &c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { c.err = std::string(what) + ": " + cudaGetErrorString(e); return SARAS_CUDA_ERROR; }
    return SARAS_OK;
}

template <int N>
static void launch_conv_n(const ConvArgs &a, cudaStream_t s) {
    int blocks = (a.nvox + 127) / 128;
    k_conv3d_tc<N><<<blocks, 128, conv_smem_bytes<N>(), s>>>(a);
}

static int launch_conv(Ctx &c, int N, const ConvArgs &a) {
    switch (N) {
    case 16: launch_conv_n<16>(a, c.stream); break;
    case 32: launch_conv_n<32>(a, c.stream); break;
    case 48: launch_conv_n<48>(a, c.stream); break;
    case 64: launch_conv_n<64>(a, c.stream); break;
    case 96: launch_conv_n<96>(a, c.stream); break;
    default: c.err = "unsupported convolution width"; return SARAS_BAD_ARG;
    }
    count_launch(c);
    return ucheck(c, "k_conv3d_tc");
}

// Activation / gradient slot indices.
enum { A_X0 = 0, A_0, A_E1, A_P1, A_2, A_E2, A_P2, A_4, A_E3, A_U2, A_6, A_F2, A_U1, A_8, A_F1, A_COUNT };

static UNet *U(Ctx &c) { return reinterpret_cast<UNet *>(c.unet); }

static int unet_alloc(Ctx &c) {
    if (c.unet) return SARAS_OK;
    UNet *u = new UNet();
    c.unet = u;
    if (c.depth < 3) { c.err = "the U-Net needs a multigrid depth of at least 3"; return SARAS_BAD_CONFIG; }
    // finest network level: the first with at most 64 intervals per axis (at
    // least level 1), keeping two coarser levels for the U-Net's depth
    int lb = 1;
    while (lb + 2 < c.depth && std::max(c.lv[lb].n[0], std::max(c.lv[lb].n[1], c.lv[lb].n[2])) > 64) ++lb;
    u->lb = lb;
    for (int q = 0; q < 3; ++q) {
        const Level &L = c.lv[lb + q];
        u->g[q] = Grid3{L.n[0] + 1, L.n[1] + 1, L.n[2] + 1};
    }
    struct Spec { int c0, c1, co, lvl; bool relu; };
    const Spec spec[11] = {{16, 0, 16, 0, true},  {16, 0, 16, 0, true},  {16, 0, 32, 1, true}, {32, 0, 32, 1, true},
                           {32, 0, 64, 2, true},  {64, 0, 64, 2, true},  {64, 32, 32, 1, true}, {32, 0, 32, 1, true},
                           {32, 16, 16, 0, true}, {16, 0, 16, 0, true},  {16, 0, 16, 0, false}};
    long off = 0;
    for (const Spec &s : spec) {
        ConvLayer l;
        l.cin0 = s.c0; l.cin1 = s.c1; l.cout = s.co; l.level = s.lvl; l.relu = s.relu;
        l.woff = off; off += 27L * (s.c0 + s.c1) * s.co;
        l.boff = off; off += s.co;
        u->flops_fwd += 2L * 27 * (s.c0 + s.c1) * s.co * u->g[s.lvl].n();
        u->L.push_back(l);
    }
    u->nparam = off;
    size_t pb = sizeof(float) * off;
    SARAS_CUDA_TRY(cudaMalloc(&u->param, pb)); SARAS_CUDA_TRY(cudaMalloc(&u->grad, pb));
    SARAS_CUDA_TRY(cudaMalloc(&u->adam_m, pb)); SARAS_CUDA_TRY(cudaMalloc(&u->adam_v, pb));
    SARAS_CUDA_TRY(cudaMemset(u->adam_m, 0, pb)); SARAS_CUDA_TRY(cudaMemset(u->adam_v, 0, pb));
    // Kaiming-uniform initialisation from a counter-based generator (seeded);
    // the output layer starts at zero so the untrained guess is the extrapolation.
    std::vector<float> h(off, 0.0f);
    uint64_t seed = (uint64_t)c.p.seed * 0x9E3779B97F4A7C15ull + 12345;
    auto rnd = [&](uint64_t i) {
        uint64_t z = seed + i * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (size_t q = 0; q < u->L.size(); ++q) {
        const ConvLayer &l = u->L[q];
        int fan = 27 * (l.cin0 + l.cin1);
        float bound = (q + 1 == u->L.size()) ? 0.0f : (float)std::sqrt(6.0 / fan);
        for (long t = 0; t < 27L * (l.cin0 + l.cin1) * l.cout; ++t) h[l.woff + t] = (float)((2.0 * rnd(l.woff + t) - 1.0) * bound);
    }
    SARAS_CUDA_TRY(cudaMemcpy(u->param, h.data(), pb, cudaMemcpyHostToDevice));
    for (ConvLayer &l : u->L) {
        size_t tiles = 27L * (l.cin0 + l.cin1) * l.cout * sizeof(bf16);
        SARAS_CUDA_TRY(cudaMalloc(&l.wf, tiles));
        SARAS_CUDA_TRY(cudaMalloc(&l.wt, tiles));
    }
    // activations (channels of each slot, level)
    const int chs[A_COUNT] = {16, 16, 16, 16, 32, 32, 32, 64, 64, 64, 32, 32, 32, 16, 16};
    const int lvl[A_COUNT] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 1, 1, 1, 0, 0, 0};
    u->act.assign(A_COUNT, nullptr);
    u->grd.assign(A_COUNT, nullptr);
    for (int s = 0; s < A_COUNT; ++s) {
        size_t bytes = sizeof(bf16) * (size_t)chs[s] * u->g[lvl[s]].n();
        SARAS_CUDA_TRY(cudaMalloc(&u->act[s], bytes));
        SARAS_CUDA_TRY(cudaMalloc(&u->grd[s], bytes));
        SARAS_CUDA_TRY(cudaMemset(u->act[s], 0, bytes));
        SARAS_CUDA_TRY(cudaMemset(u->grd[s], 0, bytes));
    }
    u->x0 = u->act[A_X0];
    long n1 = u->g[0].n();
    SARAS_CUDA_TRY(cudaMalloc(&u->out, sizeof(float) * n1));
    SARAS_CUDA_TRY(cudaMalloc(&u->feat, sizeof(float) * 4 * n1));
    SARAS_CUDA_TRY(cudaMalloc(&u->scales, sizeof(double) * 8));
    for (int q = 0; q < 3; ++q) {
        SARAS_CUDA_TRY(cudaMalloc(&u->rb[q], sizeof(double) * n1));
        SARAS_CUDA_TRY(cudaMalloc(&u->rp[q], sizeof(double) * n1));
    }
    SARAS_CUDA_TRY(cudaMalloc(&u->rpnew, sizeof(double) * n1));
    for (int q = 1; q < lb && q <= 2; ++q) {
        const Level &L = c.lv[q];
        SARAS_CUDA_TRY(cudaMalloc(&u->tmp[q - 1], sizeof(double) * (size_t)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1)));
    }
    if (lb > 3) { c.err = "grid too fine for the U-Net's restriction chain"; return SARAS_BAD_CONFIG; }
    SARAS_CUDA_TRY(cudaMalloc(&u->err, sizeof(int)));
    SARAS_CUDA_TRY(cudaMemset(u->err, 0, sizeof(int)));
    SARAS_CUDA_TRY(cudaMalloc(&u->part, sizeof(double) * std::max((n1 + 255) / 256 + 1, 2L * kAlphaBlocks)));
    u->cap = 32;
    return SARAS_OK;
}

void unet_free(Ctx &c) {
    UNet *u = U(c);
    if (!u) return;
    cudaFree(u->param); cudaFree(u->grad); cudaFree(u->adam_m); cudaFree(u->adam_v);
    for (ConvLayer &l : u->L) { cudaFree(l.wf); cudaFree(l.wt); }
    for (bf16 *p : u->act) cudaFree(p);
    for (bf16 *p : u->grd) cudaFree(p);
    for (float *p : u->samples) cudaFree(p);
    cudaFree(u->out); cudaFree(u->feat); cudaFree(u->scales); cudaFree(u->err); cudaFree(u->part);
    for (int q = 0; q < 3; ++q) { cudaFree(u->rb[q]); cudaFree(u->rp[q]); }
    cudaFree(u->rpnew); cudaFree(u->tmp[0]); cudaFree(u->tmp[1]);
    delete u;
    c.unet = nullptr;
}

int unet_create(Ctx &c) { return unet_alloc(c); }

static int pack_all(Ctx &c) {
    UNet *u = U(c);
    for (ConvLayer &l : u->L) {
        int cin = l.cin0 + l.cin1;
        long total = 27L * cin * l.cout;
        int blocks = (int)((total + 255) / 256);
        k_pack_weights<<<blocks, 256, 0, c.stream>>>(u->param + l.woff, l.wf, cin, l.cout, 0);
        k_pack_weights<<<blocks, 256, 0, c.stream>>>(u->param + l.woff, l.wt, cin, l.cout, 1);
        count_launch(c, 2);
    }
    return ucheck(c, "pack weights");
}

static ConvArgs conv_args(UNet *u, const Grid3 &g) {
    ConvArgs a;
    std::memset(&a, 0, sizeof(a));
    a.D = g.D; a.H = g.H; a.W = g.W;
    a.nvox = (int)g.n();
    a.err = u->err;
    return a;
}

static int pool(Ctx &c, const bf16 *in, bf16 *out, int C, const Grid3 &from, const Grid3 &to, bool down, float scale) {
    long total = to.n() * C;
    int blocks = (int)((total + 255) / 256);
    if (down) k_pool_down<<<blocks, 256, 0, c.stream>>>(in, out, C, from, to, scale);
    else k_pool_up<<<blocks, 256, 0, c.stream>>>(in, out, C, from, to, scale);
    count_launch(c);
    return ucheck(c, "pool");
}

// Forward pass from u->x0 to u->out (FP32 d at level 1).
static int unet_forward(Ctx &c) {
    UNet *u = U(c);
    int s;
    auto fwd = [&](int li, const bf16 *in0, const bf16 *in1, bf16 *out, float *out32) -> int {
        const ConvLayer &l = u->L[li];
        ConvArgs a = conv_args(u, u->g[l.level]);
        a.in0 = in0; a.in1 = in1; a.c0 = l.cin0; a.c1 = l.cin1;
        a.wpk = l.wf; a.bias = u->param + l.boff;
        a.out0 = out; a.split = l.cout; a.out32 = out32; a.relu = l.relu ? 1 : 0;
        prof_begin(c, PK_CONV_FWD, l.level == 0 ? 0 : 1);
        int r = launch_conv(c, l.cout, a);
        prof_end(c, PK_CONV_FWD, l.level == 0 ? 0 : 1,
                 (double)u->g[l.level].n() * 2.0 * (l.cin0 + l.cin1 + l.cout));
        return r;
    };
    auto A = [&](int q) { return u->act[q]; };
    if ((s = fwd(0, A(A_X0), nullptr, A(A_0), nullptr))) return s;
    if ((s = fwd(1, A(A_0), nullptr, A(A_E1), nullptr))) return s;
    if ((s = pool(c, A(A_E1), A(A_P1), 16, u->g[0], u->g[1], true, 1.0f))) return s;
    if ((s = fwd(2, A(A_P1), nullptr, A(A_2), nullptr))) return s;
    if ((s = fwd(3, A(A_2), nullptr, A(A_E2), nullptr))) return s;
    if ((s = pool(c, A(A_E2), A(A_P2), 32, u->g[1], u->g[2], true, 1.0f))) return s;
    if ((s = fwd(4, A(A_P2), nullptr, A(A_4), nullptr))) return s;
    if ((s = fwd(5, A(A_4), nullptr, A(A_E3), nullptr))) return s;
    if ((s = pool(c, A(A_E3), A(A_U2), 64, u->g[2], u->g[1], false, 1.0f))) return s;
    if ((s = fwd(6, A(A_U2), A(A_E2), A(A_6), nullptr))) return s;
    if ((s = fwd(7, A(A_6), nullptr, A(A_F2), nullptr))) return s;
    if ((s = pool(c, A(A_F2), A(A_U1), 32, u->g[1], u->g[0], false, 1.0f))) return s;
    if ((s = fwd(8, A(A_U1), A(A_E1), A(A_8), nullptr))) return s;
    if ((s = fwd(9, A(A_8), nullptr, A(A_F1), nullptr))) return s;
    if ((s = fwd(10, A(A_F1), nullptr, nullptr, u->out))) return s;
    return SARAS_OK;
}

static int add_mask(Ctx &c, const bf16 *a, const bf16 *b, const bf16 *mask, bf16 *out, long n) {
    k_add_mask<<<(int)((n + 255) / 256), 256, 0, c.stream>>>(a, b, mask, out, n);
    count_launch(c);
    return ucheck(c, "add_mask");
}

// Weight and bias gradients of layer li on the tensor cores (k_conv_dw_tc):
// voxel chunks sized for about four CTAs an SM over all M tiles.
template <int N>
static cudaError_t launch_dw_n(const DwArgs &a, int mtiles, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_dw_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, dw_smem_bytes<N>());
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long nch = (a.nvox + a.chunk - 1) / a.chunk;
    k_conv_dw_tc<N><<<dim3((unsigned)nch, (unsigned)mtiles), 128, dw_smem_bytes<N>(), st>>>(a);
    return cudaGetLastError();
}

static int launch_dw(Ctx &c, int N, DwArgs a) {
    const int cin = a.c0 + a.c1;
    const int mtiles = (27 * cin + 127) / 128;
    const long want = std::max(1L, 4L * 152 / mtiles);   // voxel chunks
    a.chunk = (int)std::max(16L, (((long)a.nvox + want - 1) / want + 15) / 16 * 16);
    cudaError_t e;
    switch (N) {
    case 16: e = launch_dw_n<16>(a, mtiles, c.stream); break;
    case 32: e = launch_dw_n<32>(a, mtiles, c.stream); break;
    case 48: e = launch_dw_n<48>(a, mtiles, c.stream); break;
    case 64: e = launch_dw_n<64>(a, mtiles, c.stream); break;
    case 96: e = launch_dw_n<96>(a, mtiles, c.stream); break;
    default: c.err = "unsupported convolution width"; return SARAS_BAD_ARG;
    }
    count_launch(c);
    if (e != cudaSuccess) { c.err = std::string("k_conv_dw_tc: ") + cudaGetErrorString(e); return SARAS_CUDA_ERROR; }
    return SARAS_OK;
}

static int conv_dw(Ctx &c, int li, const bf16 *x0, const bf16 *x1, const bf16 *dy) {
    UNet *u = U(c);
    const ConvLayer &l = u->L[li];
    const Grid3 &g = u->g[l.level];
    DwArgs a;
    a.in0 = x0; a.in1 = x1; a.c0 = l.cin0; a.c1 = l.cin1;
    a.dy = dy;
    a.dw = u->grad + l.woff;
    a.db = u->grad + l.boff;
    a.D = g.D; a.H = g.H; a.W = g.W; a.nvox = (int)g.n();
    a.chunk = 0;
    a.err = u->err;
    return launch_dw(c, l.cout, a);
}

// Input gradient of layer li: conv of dY with the mirrored, transposed weights.
static int conv_dx(Ctx &c, int li, const bf16 *dy, bf16 *out0, bf16 *out1, const bf16 *mask0) {
    UNet *u = U(c);
    const ConvLayer &l = u->L[li];
    ConvArgs a = conv_args(u, u->g[l.level]);
    a.in0 = dy; a.c0 = l.cout; a.in1 = nullptr; a.c1 = 0;
    a.wpk = l.wt; a.bias = nullptr; a.relu = 0;
    a.out0 = out0; a.out1 = out1; a.split = l.cin1 ? l.cin0 : l.cin0;
    a.mask0 = mask0;
    prof_begin(c, PK_CONV_BWD, l.level == 0 ? 0 : 1);
    int s = launch_conv(c, l.cin0 + l.cin1, a);
    prof_end(c, PK_CONV_BWD, l.level == 0 ? 0 : 1, (double)u->g[l.level].n() * 2.0 * (l.cin0 + l.cin1 + l.cout));
    return s;
}

// Backward pass from the output gradient in grd[A_F1]-shaped buffer `gout`.
static int unet_backward(Ctx &c, const bf16 *gout) {
    UNet *u = U(c);
    int s;
    auto A = [&](int q) { return u->act[q]; };
    auto G = [&](int q) { return u->grd[q]; };
    long n1 = u->g[0].n(), n2 = u->g[1].n(), n3 = u->g[2].n();
    SARAS_CUDA_TRY(cudaMemsetAsync(u->grad, 0, sizeof(float) * u->nparam, c.stream));
    // layer 10 (no ReLU): dW, dX masked by f1 > 0 -> dY9
    if ((s = conv_dw(c, 10, A(A_F1), nullptr, gout))) return s;
    if ((s = conv_dx(c, 10, gout, G(A_F1), nullptr, A(A_F1)))) return s;
    if ((s = conv_dw(c, 9, A(A_8), nullptr, G(A_F1)))) return s;
    if ((s = conv_dx(c, 9, G(A_F1), G(A_8), nullptr, A(A_8)))) return s;
    // layer 8: input concat(u1 32, e1 16)
    if ((s = conv_dw(c, 8, A(A_U1), A(A_E1), G(A_8)))) return s;
    if ((s = conv_dx(c, 8, G(A_8), G(A_U1), G(A_0), nullptr))) return s;   // G(A_0) holds de1 (skip path)
    // up1 backward: dF2 = 8 * down(dU1), masked by f2
    if ((s = pool(c, G(A_U1), G(A_F2), 32, u->g[0], u->g[1], true, 8.0f))) return s;
    if ((s = add_mask(c, G(A_F2), nullptr, A(A_F2), G(A_F2), n2 * 32))) return s;
    if ((s = conv_dw(c, 7, A(A_6), nullptr, G(A_F2)))) return s;
    if ((s = conv_dx(c, 7, G(A_F2), G(A_6), nullptr, A(A_6)))) return s;
    // layer 6: input concat(u2 64, e2 32)
    if ((s = conv_dw(c, 6, A(A_U2), A(A_E2), G(A_6)))) return s;
    if ((s = conv_dx(c, 6, G(A_6), G(A_U2), G(A_2), nullptr))) return s;    // G(A_2) holds de2 (skip path)
    // up2 backward: dE3 = 8 * down(dU2), masked by e3
    if ((s = pool(c, G(A_U2), G(A_E3), 64, u->g[1], u->g[2], true, 8.0f))) return s;
    if ((s = add_mask(c, G(A_E3), nullptr, A(A_E3), G(A_E3), n3 * 64))) return s;
    if ((s = conv_dw(c, 5, A(A_4), nullptr, G(A_E3)))) return s;
    if ((s = conv_dx(c, 5, G(A_E3), G(A_4), nullptr, A(A_4)))) return s;
    if ((s = conv_dw(c, 4, A(A_P2), nullptr, G(A_4)))) return s;
    if ((s = conv_dx(c, 4, G(A_4), G(A_P2), nullptr, nullptr))) return s;
    // pool2 backward: dE2 += up(dP2) / 8; then mask by e2
    if ((s = pool(c, G(A_P2), G(A_E2), 32, u->g[2], u->g[1], false, 0.125f))) return s;
    if ((s = add_mask(c, G(A_E2), G(A_2), A(A_E2), G(A_E2), n2 * 32))) return s;
    if ((s = conv_dw(c, 3, A(A_2), nullptr, G(A_E2)))) return s;
    if ((s = conv_dx(c, 3, G(A_E2), G(A_2), nullptr, A(A_2)))) return s;
    if ((s = conv_dw(c, 2, A(A_P1), nullptr, G(A_2)))) return s;
    if ((s = conv_dx(c, 2, G(A_2), G(A_P1), nullptr, nullptr))) return s;
    // pool1 backward: dE1 = up(dP1) / 8 + de1 (skip), masked by e1
    if ((s = pool(c, G(A_P1), G(A_E1), 16, u->g[1], u->g[0], false, 0.125f))) return s;
    if ((s = add_mask(c, G(A_E1), G(A_0), A(A_E1), G(A_E1), n1 * 16))) return s;
    if ((s = conv_dw(c, 1, A(A_0), nullptr, G(A_E1)))) return s;
    if ((s = conv_dx(c, 1, G(A_E1), G(A_0), nullptr, A(A_0)))) return s;
    if ((s = conv_dw(c, 0, A(A_X0), nullptr, G(A_0)))) return s;
    return SARAS_OK;
}

static L0View l0view(const Ctx &c, const double *p) {
    L0View v;
    v.p = p;
    for (int d = 0; d < 3; ++d) v.n[d] = c.lv[0].n[d];
    return v;
}

static int ensure_hist(Ctx &c) {
    if (c.pHist[0]) return SARAS_OK;
    size_t bytes = sizeof(double) * c.lv[0].count;
    for (int q = 0; q < 3; ++q) {
        SARAS_CUDA_TRY(cudaMalloc(&c.pHist[q], bytes));
        SARAS_CUDA_TRY(cudaMemsetAsync(c.pHist[q], 0, bytes, c.stream));
    }
    return SARAS_OK;
}

// R^lb of a level-0 padded field into dst (a level-lb core array).
static int restrict_to_base(Ctx &c, const double *src, double *dst) {
    UNet *u = U(c);
    const Level &L1 = c.lv[1];
    Grid3 g1{L1.n[0] + 1, L1.n[1] + 1, L1.n[2] + 1};
    double *first = u->lb == 1 ? dst : u->tmp[0];
    k_restrict0<<<dim3((g1.W + 31) / 32, (g1.H + 7) / 8, (g1.D + kR0Ch - 1) / kR0Ch), dim3(32, 8, 1), 0, c.stream>>>(l0view(c, src), g1,
                                                                                                                 first);
    count_launch(c);
    Grid3 gf = g1;
    for (int l = 2; l <= u->lb; ++l) {
        const Level &L = c.lv[l];
        Grid3 gc{L.n[0] + 1, L.n[1] + 1, L.n[2] + 1};
        const double *in = u->tmp[l - 2];
        double *out = l == u->lb ? dst : u->tmp[l - 1];
        k_restrict<<<(int)((gc.n() + 255) / 256), 256, 0, c.stream>>>(in, gf, gc, out);
        count_launch(c);
        gf = gc;
    }
    return ucheck(c, "restrict");
}

// rb ring: this solve's R b (once per solve, in the solves that keep the rings).
static int push_b(Ctx &c, const double *b) {
    UNet *u = U(c);
    if (!u->track || u->bPushed) return SARAS_OK;
    std::swap(u->rb[2], u->rb[1]);
    std::swap(u->rb[1], u->rb[0]);
    u->nb += 1;
    u->bPushed = true;
    return restrict_to_base(c, b, u->rb[0]);
}

// Scales and features of this solve at level lb (target from rpnew when given).
static int features(Ctx &c, float *feat, float *target) {
    UNet *u = U(c);
    long n = u->g[0].n();
    SARAS_CUDA_TRY(cudaMemsetAsync(u->scales, 0, sizeof(double) * 3, c.stream));
    k_feat_scales<<<152, 256, 0, c.stream>>>(u->rb[0], u->rb[1], u->rb[2], u->rp[0], u->rp[1], n, u->scales);
    double lfac = (c.p.Lx * c.p.Lx + c.p.Ly * c.p.Ly + c.p.Lz * c.p.Lz) / (3.0 * 4.0 * M_PI * M_PI);
    k_floor_scale<<<1, 32, 0, c.stream>>>(u->scales, 1e-300, lfac);
    k_features<<<(int)((n + 255) / 256), 256, 0, c.stream>>>(u->rb[0], u->rb[1], u->rb[2], u->rp[0], u->rp[1], u->rpnew, n, u->scales,
                                                             feat, target);
    count_launch(c, 3);
    return ucheck(c, "features");
}

}  // namespace saras

// ------------------------------------------------------------------ solver hooks
namespace saras {

// Whether this solve keeps the restricted histories.  The network's inputs
// are R b of this and the two previous solves and R Pp of the two previous
// ones, so the rings run while pairs are collected and in the solves leading
// up to any solve that may use the network: its first uses, while it is
// preferred, after a pick that found the rings incomplete, and from two solves
// before a scheduled probe of it.  Elsewhere the learned mode costs what
// extrapolation costs.
static bool rings_due(const Ctx &c, const UNet *u) {
    if (c.collecting) return true;
    if (c.guessMode == SARAS_GUESS_NETWORK) return u->trained;
    if (c.guessMode != SARAS_GUESS_LEARNED || !u->trained) return false;
    if (u->wantNet || u->usesNet < 2 || u->usesExt < 2 || u->preferNet) return true;
    return u->nextProbe > 0 && u->solves + 3 >= u->nextProbe;
}

// Whether this solve pushes R b (the FP64 b must then be stored).
bool unet_tracking(const Ctx &c) {
    const UNet *u = reinterpret_cast<const UNet *>(c.unet);
    return u && u->track;
}

// Called at the start of a target-mode solve: rotate the pressure history
// (and, in the solves that keep them, its restriction to level lb).  When Pp
// and a history buffer have one size, the rotation moves buffers instead of
// copying: Pp's buffer (P of the last solve) becomes pHist[0] and the oldest
// history buffer becomes Pp, which the solve then writes in full; until it
// does, the previous Pp is pHist[0] (c.ppInHist).
int unet_begin_solve(Ctx &c) {
    int s = ensure_hist(c);
    if (s) return s;
    double *oldest = c.pHist[2];
    c.pHist[2] = c.pHist[1];
    c.pHist[1] = c.pHist[0];
    const FieldInfo &fp = c.info[SARAS_FIELD_PP];
    const Level &L0 = c.lv[0];
    if (fp.n[0] + 2 == L0.n[0] + 3 && fp.n[1] + 2 == L0.n[1] + 3 && fp.n[2] + 2 == L0.n[2] + 3) {   // one padded shape
        c.pHist[0] = c.f[SARAS_FIELD_PP];
        c.f[SARAS_FIELD_PP] = oldest;
        c.ppInHist = true;
    } else {
        c.pHist[0] = oldest;
        SARAS_CUDA_TRY(cudaMemcpyAsync(c.pHist[0], c.f[SARAS_FIELD_PP], sizeof(double) * c.lv[0].count, cudaMemcpyDeviceToDevice,
                                       c.stream));
    }
    c.histCount += 1;
    UNet *u = U(c);
    if (!u) return SARAS_OK;
    u->bPushed = false;
    u->track = rings_due(c, u);
    if (!u->track) {
        u->np = u->nb = 0;   // the restricted histories are no longer consecutive
        return SARAS_OK;
    }
    std::swap(u->rp[2], u->rp[1]);
    std::swap(u->rp[1], u->rp[0]);
    u->np += 1;
    return restrict_to_base(c, c.pHist[0], u->rp[0]);
}

// SARAS_GUESS_LEARNED picks, per solve, between the network's guess and plain
// extrapolation by the residual each leaves (moving averages of its log10
// over recent solves: the V-cycles a solve needs follow it, about one a
// decade).  Building the network's guess costs about half a level-0 V-cycle
// more than extrapolating (restrictions, features, forward pass), so the
// network is preferred when its average is lower by more than half a decade.
// The other guess is probed so that its average stays current: first after
// kProbe solves, then at doubling intervals up to kProbeMax while the
// preference holds (back to kProbe when it changes).  A probe, and each of the
// first two uses of either guess, builds both guesses (unet_shadow) and the
// better one starts the solve, so probing a worse guess costs its building
// and one residual pass, not V-cycles.
constexpr int kProbe = 8, kProbeMax = 64;
constexpr double kNetCostDecades = 0.5;

int unet_pick(Ctx &c) {
    UNet *u = U(c);
    if (c.guessMode == SARAS_GUESS_NETWORK) {   // the network whenever its histories are complete
        if (!u || !u->trained) return SARAS_GUESS_EXTRAPOLATE;
        return u->track && u->nb >= 2 && u->np >= 2 ? SARAS_GUESS_LEARNED : SARAS_GUESS_EXTRAPOLATE;
    }
    if (c.guessMode != SARAS_GUESS_LEARNED) return c.guessMode;
    if (!u || !u->trained) return SARAS_GUESS_EXTRAPOLATE;
    u->solves += 1;
    u->shadow = false;
    bool net, probe = false;
    if (u->usesNet < 2 || u->usesExt < 2) {
        net = u->usesNet < 2;
        u->shadow = true;
    } else {
        bool netBetter = u->lrNet + kNetCostDecades < u->lrExt;
        if (u->nextProbe == 0) u->nextProbe = u->solves + kProbe;   // the first comparison starts the schedule
        if (netBetter != u->preferNet) {
            u->preferNet = netBetter;
            u->probeEvery = kProbe;
            u->nextProbe = u->solves + kProbe;
        }
        probe = u->solves >= u->nextProbe;
        net = netBetter;
        u->shadow = probe;
    }
    // the rings are complete once this solve pushes its R b
    const bool ready = u->track && u->nb >= 2 && u->np >= 2;
    if ((net || u->shadow) && !ready) {
        u->wantNet = true;   // they run from the next solve on; the pick (a probe too) waits for them
        u->shadow = false;
        return SARAS_GUESS_EXTRAPOLATE;
    }
    u->wantNet = false;
    if (probe) {
        u->nextProbe = u->solves + u->probeEvery;
        u->probeEvery = std::min(kProbeMax, 2 * u->probeEvery);
    }
    return net ? SARAS_GUESS_LEARNED : SARAS_GUESS_EXTRAPOLATE;
}

// The guess this solve also builds beside `built` (0: none).
int unet_shadow(Ctx &c, int built) {
    UNet *u = U(c);
    if (!u || c.guessMode != SARAS_GUESS_LEARNED || !u->shadow) return 0;
    u->shadow = false;
    return built == SARAS_GUESS_LEARNED ? SARAS_GUESS_EXTRAPOLATE : SARAS_GUESS_LEARNED;
}

// The residual (relative to max|b|) that guess `built` left at the start of a solve.
void unet_note_start(Ctx &c, int built, double rel) {
    UNet *u = U(c);
    if (!u || c.guessMode != SARAS_GUESS_LEARNED || !(rel > 0.0) || !std::isfinite(rel)) return;
    const double w = 0.3, lr = std::log10(rel);
    if (built == SARAS_GUESS_LEARNED) {
        u->lrNet = u->usesNet ? (1.0 - w) * u->lrNet + w * lr : lr;
        u->usesNet += 1;
    } else if (built == SARAS_GUESS_EXTRAPOLATE) {
        u->lrExt = u->usesExt ? (1.0 - w) * u->lrExt + w * lr : lr;
        u->usesExt += 1;
    }
}

// Build the learned (or extrapolated) guess for the level-0 iterate into `dst`,
// or with fxdst into the fixed-point iterate fxdst (round(v 2^sc), flag set
// when out of range); b is the compatible right-hand side.  Returns
// BAD_CONFIG if unavailable.
int unet_guess(Ctx &c, const double *b, double *dst, int mode, long long *fxdst, int sc, int *flag) {
    bool use_net = mode == SARAS_GUESS_LEARNED;
    int quad = mode == SARAS_GUESS_QUADRATIC ? 1 : mode == SARAS_GUESS_PARITY ? 2 : 0;
    if (c.histCount < 2 + (quad ? 1 : 0)) return SARAS_BAD_CONFIG;
    int s;
    UNet *u = U(c);
    if ((c.guessMode == SARAS_GUESS_LEARNED || c.guessMode == SARAS_GUESS_NETWORK) && u && u->trained && (s = push_b(c, b))) return s;
    if (use_net) {
        if (!u || !u->trained) return SARAS_BAD_CONFIG;
        if (u->nb < 3 || u->np < 2) use_net = false;   // histories not yet consecutive: plain extrapolation
    }
    if (use_net) {
        long n = u->g[0].n();
        if ((s = features(c, u->feat, nullptr))) return s;
        k_expand<<<(int)((n * 16 + 255) / 256), 256, 0, c.stream>>>(u->feat, u->x0, n);
        count_launch(c);
        if ((s = unet_forward(c))) return s;
        // two low-pass passes (out -> feat -> out; feat is free after the forward pass)
        k_lowpass<<<(int)((n + 255) / 256), 256, 0, c.stream>>>(u->out, u->feat, u->g[0]);
        k_lowpass<<<(int)((n + 255) / 256), 256, 0, c.stream>>>(u->feat, u->out, u->g[0]);
        const Level &Lb = c.lv[u->lb];
        k_alpha_coarse<<<kAlphaBlocks, 256, 0, c.stream>>>(u->out, u->rb[0], u->rb[1], u->rb[2], u->g[0], c.p.xPer, c.p.yPer, c.p.zPer,
                                                           Lb.lx, Lb.ly, Lb.lz, u->scales, u->part);
        k_alpha_final<<<1, 32, 0, c.stream>>>(u->part, kAlphaBlocks, u->scales + 4);
        count_launch(c, 4);
    }
    const Level &L0 = c.lv[0];
    dim3 b2(256), g2((unsigned)(((long)(L0.n[1] + 1) * (L0.n[2] + 1) + 255) / 256), 1, L0.n[0] + 1);
    const float *d = use_net ? u->out : nullptr;
    Grid3 gd = use_net ? u->g[0] : Grid3{1, 1, 1};
    int lb = use_net ? u->lb : 0;
    const double *sca = use_net ? u->scales : nullptr, *alpha = use_net ? u->scales + 4 : nullptr;
    if (fxdst)
        k_apply_guess<long long><<<g2, b2, 0, c.stream>>>(fxdst, l0view(c, c.pHist[0]), l0view(c, c.pHist[1]), l0view(c, c.pHist[2]), quad,
                                                          d, gd, lb, sca, alpha, c.p.xPer, c.p.yPer, c.p.zPer, sc, flag);
    else
        k_apply_guess<double><<<g2, b2, 0, c.stream>>>(dst, l0view(c, c.pHist[0]), l0view(c, c.pHist[1]), l0view(c, c.pHist[2]), quad,
                                                       d, gd, lb, sca, alpha, c.p.xPer, c.p.yPer, c.p.zPer, 0, nullptr);
    count_launch(c);
    return ucheck(c, "guess");
}

// After a solve that reached the target: one training pair (features of this
// solve, target R(P_new - (2 P1 - P2))).
int unet_collect_sample(Ctx &c, const double *b) {
    int s = unet_alloc(c);
    if (s) return s;
    UNet *u = U(c);
    if ((s = push_b(c, b))) return s;
    // the first solves of a run are the start-up transient of the pressure
    // correction; pairs are taken once two earlier corrections exist beyond it
    if (c.histCount < 4 || u->nb < 3 || u->np < 2) return SARAS_OK;
    long n = u->g[0].n();
    float *dst;
    if (u->nsamples < u->cap) {
        SARAS_CUDA_TRY(cudaMalloc(&dst, sizeof(float) * 4 * n));
        u->samples.push_back(dst);
        u->nsamples += 1;
    } else {
        dst = u->samples[u->next];
        u->next = (u->next + 1) % u->cap;
    }
    if ((s = restrict_to_base(c, c.f[SARAS_FIELD_PP], u->rpnew))) return s;
    if ((s = features(c, dst, dst + 3 * n))) return s;
    return ucheck(c, "collect");
}

int unet_collect(Ctx &c) {
    int s = unet_alloc(c);
    if (s) return s;
    c.collecting = true;
    return SARAS_OK;
}

int unet_train(Ctx &c, int iters, double lr, double *loss) {
    int s = unet_alloc(c);
    if (s) return s;
    UNet *u = U(c);
    c.collecting = false;
    if (u->nsamples == 0) { c.err = "no training pairs collected"; return SARAS_BAD_CONFIG; }
    long n1 = u->g[0].n();
    int nb = (int)((n1 + 255) / 256);
    double last = 0.0;
    SARAS_CUDA_TRY(cudaMemsetAsync(u->err, 0, sizeof(int), c.stream));
    for (int it = 0; it < iters; ++it) {
        if ((s = pack_all(c))) return s;
        const float *smp = u->samples[it % u->nsamples];
        k_expand<<<(int)((n1 * 16 + 255) / 256), 256, 0, c.stream>>>(smp, u->x0, n1);
        count_launch(c);
        if ((s = unet_forward(c))) return s;
        k_loss<<<nb, 256, 0, c.stream>>>(u->out, smp + 3 * n1, u->grd[A_X0], n1, u->part);
        count_launch(c);
        if (it == iters - 1) {
            k_final_reduce<<<1, 256, 0, c.stream>>>(u->part, nb, 0, u->scales + 3);
            count_launch(c);
        }
        if ((s = unet_backward(c, u->grd[A_X0]))) return s;
        u->adam_t += 1;
        float b1 = 0.9f, b2 = 0.999f;
        float c1 = 1.0f - std::pow(b1, (float)u->adam_t), c2 = 1.0f - std::pow(b2, (float)u->adam_t);
        k_adam<<<(int)((u->nparam + 255) / 256), 256, 0, c.stream>>>(u->param, u->grad, u->adam_m, u->adam_v, u->nparam, (float)lr, b1, b2,
                                                                      1e-8f, c1, c2);
        count_launch(c);
    }
    if ((s = pack_all(c))) return s;
    int herr = 0;
    SARAS_CUDA_TRY(cudaMemcpyAsync(&herr, u->err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaMemcpyAsync(&last, u->scales + 3, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (herr) { c.err = "tensor-core convolution timed out waiting on an mbarrier"; return SARAS_CUDA_ERROR; }
    u->trained = true;
    if (loss) *loss = last;
    return SARAS_OK;
}

// The network's parameter count and finest grid (the voxels of one sample).
int unet_shape(Ctx &c, long long *nparam, int dims[3]) {
    int s = unet_alloc(c);
    if (s) return s;
    UNet *u = U(c);
    if (nparam) *nparam = u->nparam;
    if (dims) { dims[0] = u->g[0].D; dims[1] = u->g[0].H; dims[2] = u->g[0].W; }
    return SARAS_OK;
}

// One training step's forward and backward pass without the update: the
// features (nvox x 3, channels last) and target (nvox) of a sample, the
// parameters (nparam, or null for the current ones) in; the output d (nvox),
// loss 0.5 mean (d - target)^2 and its gradient with respect to every
// parameter out.  The kernels are those of unet_train.
int unet_grad_check(Ctx &c, const float *feat, const float *target, const float *params, float *out, double *loss, float *grad) {
    int s = unet_alloc(c);
    if (s) return s;
    UNet *u = U(c);
    const long n1 = u->g[0].n();
    const int nb = (int)((n1 + 255) / 256);
    if (params) SARAS_CUDA_TRY(cudaMemcpyAsync(u->param, params, sizeof(float) * u->nparam, cudaMemcpyHostToDevice, c.stream));
    SARAS_CUDA_TRY(cudaMemcpyAsync(u->feat, feat, sizeof(float) * 3 * n1, cudaMemcpyHostToDevice, c.stream));
    SARAS_CUDA_TRY(cudaMemcpyAsync(u->feat + 3 * n1, target, sizeof(float) * n1, cudaMemcpyHostToDevice, c.stream));
    SARAS_CUDA_TRY(cudaMemsetAsync(u->err, 0, sizeof(int), c.stream));
    if ((s = pack_all(c))) return s;
    k_expand<<<(int)((n1 * 16 + 255) / 256), 256, 0, c.stream>>>(u->feat, u->x0, n1);
    count_launch(c);
    if ((s = unet_forward(c))) return s;
    k_loss<<<nb, 256, 0, c.stream>>>(u->out, u->feat + 3 * n1, u->grd[A_X0], n1, u->part);
    k_final_reduce<<<1, 256, 0, c.stream>>>(u->part, nb, 0, u->scales + 3);
    count_launch(c, 2);
    if ((s = unet_backward(c, u->grd[A_X0]))) return s;
    double sum = 0.0;
    int herr = 0;
    if (out) SARAS_CUDA_TRY(cudaMemcpyAsync(out, u->out, sizeof(float) * n1, cudaMemcpyDeviceToHost, c.stream));
    if (grad) SARAS_CUDA_TRY(cudaMemcpyAsync(grad, u->grad, sizeof(float) * u->nparam, cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaMemcpyAsync(&sum, u->scales + 3, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaMemcpyAsync(&herr, u->err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (herr) { c.err = "tensor-core convolution timed out waiting on an mbarrier"; return SARAS_CUDA_ERROR; }
    if (loss) *loss = sum / (double)n1;
    return ucheck(c, "unet grad check");
}

// The learned guess for the current right-hand side into `out` (history and
// the level-lb rings as the next solve would see them; no rotation).
int unet_infer(Ctx &c, double *out) {
    return unet_guess(c, c.lv[0].r, out, SARAS_GUESS_LEARNED);
}

}  // namespace saras

// ------------------------------------------------------------------ stand-alone convolution check
namespace saras {

__global__ void k_bf16_to_f32(const bf16 *a, float *b, long n) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t < n) b[t] = __bfloat162float(a[t]);
}

int conv3d_check(int mode, int D, int H, int W, int cin, int cout, const unsigned short *x, const unsigned short *dy,
                 const float *w, const float *bias, int relu, float *out) {
    if (D < 1 || H < 1 || W < 1 || cin % 16 || cout % 16 || cin < 16 || cout < 16 || cin > 96 || cout > 96) return SARAS_BAD_ARG;
    if ((long)D * H * W > (1L << 24)) return SARAS_TOO_LARGE;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); set_error("no CUDA device"); return SARAS_NO_DEVICE; }
    Ctx c;   // scratch context: stream + launch accounting only
    c.stream = 0;
    long nv = (long)D * H * W;
    bf16 *dx = nullptr, *ddy = nullptr, *dout = nullptr, *wf = nullptr, *wt = nullptr;
    float *dw = nullptr, *dbias = nullptr, *dgrad = nullptr, *dout32 = nullptr;
    int *derr = nullptr;
    int s = SARAS_OK;
    auto fail = [&](cudaError_t e) { set_error(cudaGetErrorString(e)); s = SARAS_CUDA_ERROR; };
    cudaError_t e;
    size_t wbytes = sizeof(float) * 27L * cin * cout;
    if ((e = cudaMalloc(&dx, sizeof(bf16) * nv * cin)) || (e = cudaMalloc(&ddy, sizeof(bf16) * nv * cout)) ||
        (e = cudaMalloc(&dout, sizeof(bf16) * nv * std::max(cin, cout))) || (e = cudaMalloc(&wf, sizeof(bf16) * 27L * cin * cout)) ||
        (e = cudaMalloc(&wt, sizeof(bf16) * 27L * cin * cout)) || (e = cudaMalloc(&dw, wbytes)) || (e = cudaMalloc(&dbias, sizeof(float) * cout)) ||
        (e = cudaMalloc(&dgrad, wbytes + sizeof(float) * cout)) || (e = cudaMalloc(&dout32, sizeof(float) * nv * std::max(cin, cout))) ||
        (e = cudaMalloc(&derr, sizeof(int)))) {
        fail(e);
    }
    if (!s) {
        cudaMemset(derr, 0, sizeof(int));
        if (x) cudaMemcpy(dx, x, sizeof(bf16) * nv * cin, cudaMemcpyHostToDevice);
        else cudaMemset(dx, 0, sizeof(bf16) * nv * cin);
        if (dy) cudaMemcpy(ddy, dy, sizeof(bf16) * nv * cout, cudaMemcpyHostToDevice);
        else cudaMemset(ddy, 0, sizeof(bf16) * nv * cout);
        cudaMemcpy(dw, w, wbytes, cudaMemcpyHostToDevice);
        if (bias) cudaMemcpy(dbias, bias, sizeof(float) * cout, cudaMemcpyHostToDevice);
        else cudaMemset(dbias, 0, sizeof(float) * cout);
        long total = 27L * cin * cout;
        k_pack_weights<<<(int)((total + 255) / 256), 256>>>(dw, wf, cin, cout, 0);
        k_pack_weights<<<(int)((total + 255) / 256), 256>>>(dw, wt, cin, cout, 1);
        ConvArgs a;
        std::memset(&a, 0, sizeof(a));
        a.D = D; a.H = H; a.W = W; a.nvox = (int)nv; a.err = derr;
        if (mode == 0) {
            a.in0 = dx; a.c0 = cin; a.wpk = wf; a.bias = dbias; a.out0 = dout; a.split = cout; a.relu = relu;
            s = launch_conv(c, cout, a);
            if (!s) k_bf16_to_f32<<<(int)((nv * cout + 255) / 256), 256>>>(dout, dout32, nv * cout);
            if (!s && (e = cudaMemcpy(out, dout32, sizeof(float) * nv * cout, cudaMemcpyDeviceToHost))) fail(e);
        } else if (mode == 1) {
            a.in0 = ddy; a.c0 = cout; a.wpk = wt; a.out0 = dout; a.split = cin;
            s = launch_conv(c, cin, a);
            if (!s) k_bf16_to_f32<<<(int)((nv * cin + 255) / 256), 256>>>(dout, dout32, nv * cin);
            if (!s && (e = cudaMemcpy(out, dout32, sizeof(float) * nv * cin, cudaMemcpyDeviceToHost))) fail(e);
        } else if (mode == 2) {
            cudaMemset(dgrad, 0, wbytes + sizeof(float) * cout);
            DwArgs da;
            da.in0 = dx; da.in1 = nullptr; da.c0 = cin; da.c1 = 0;
            da.dy = ddy; da.dw = dgrad; da.db = dgrad + 27L * cin * cout;
            da.D = D; da.H = H; da.W = W; da.nvox = (int)nv; da.chunk = 0; da.err = derr;
            s = launch_dw(c, cout, da);
            if (!s && (e = cudaMemcpy(out, dgrad, wbytes + sizeof(float) * cout, cudaMemcpyDeviceToHost))) fail(e);
        } else {
            s = SARAS_BAD_ARG;
        }
        int herr = 0;
        if (!s && (e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost))) fail(e);
        if (!s && herr) { set_error("tensor-core convolution timed out on an mbarrier"); s = SARAS_CUDA_ERROR; }
        if (!s && (e = cudaDeviceSynchronize())) fail(e);
    }
    cudaFree(dx); cudaFree(ddy); cudaFree(dout); cudaFree(wf); cudaFree(wt); cudaFree(dw); cudaFree(dbias);
    cudaFree(dgrad); cudaFree(dout32); cudaFree(derr);
    return s;
}

}  // namespace saras

extern "C" int saras_conv3d_check(int mode, int D, int H, int W, int cin, int cout, const unsigned short *x,
                                  const unsigned short *dy, const float *w, const float *bias, int relu, float *out) {
    return saras::conv3d_check(mode, D, H, W, cin, cout, x, dy, w, bias, relu, out);
}
