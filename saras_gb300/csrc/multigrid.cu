// multigrid.cu -- geometric multigrid for the pressure-correction Poisson
// equation (lib/poisson/poisson.cc, poisson_d3.cc) on one GB300.
//
// Three modes share one set of templated level kernels:
//   SARAS_MG_REFERENCE     FP64, the reference V-cycle loop bit for bit
//                          (padded-array mean removal, |delta residual| stop,
//                          coarsest Gauss-Seidel to mgTolerance / maxCount).
//   SARAS_MG_PLAIN_TARGET  FP64 V-cycles on the compatible system until
//                          max|b-Ap| <= target * max|b|.
//   SARAS_MG_MIXED         FP32 V-cycles as the inner solver of an
//                          iterative-refinement loop to the same target; the
//                          outer residual is FP64, or exact 64-bit fixed point
//                          when the level-0 stencil is isotropic (k_fx_refine).
// The target modes make the singular Neumann/periodic system compatible by
// subtracting the trapezoidal-weight mean of b (the left null vector of the
// vertex-grid operator with mirror or periodic ghosts) and use a damped Jacobi
// smoother; they exist for the throughput comparison and are not drop-ins.
//
// Ghost handling: in the reference mode the smoother and prolongation write
// every face-ghost image of the points they produce (imposeBC,
// poisson_d3.cc:575-668, restricted to the face ghosts a 7-point stencil
// reads), and the restriction resolves the pads of the residual array
// (updatePads, poisson_d3.cc:671-686) by index mapping.  The target-mode level
// kernels resolve every face neighbour by index mapping (pad_img, nbr_jk) and
// write the core only.
// Compiled with --fmad=false (see fields.cu).

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <algorithm>

#include "context.cuh"
#include "df64.cuh"
#include <utility>
#include "tma.cuh"

#include <cudaTypedefs.h>

namespace saras {

__global__ void k_final_reduce(const double *part, int n, int op, double *out);

// max |a| over a whole array into *out (non-negative, atomic).
__global__ void k_maxabs(const double *a, long n, double *out) {
    double m = 0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) m = fmax(m, fabs(a[t]));
    block_max_to(m, out);
}

// Deterministic sums in the oracle's chunked order: thread t sums elements
// [t*4096, (t+1)*4096) in index order; one thread then sums the chunk sums in
// chunk order.  mode 0: a[t] over a flat array; mode 1/2: |Lap(p)-r|^2 / r^2
// over the level-0 core (computeError norm 2).
constexpr long kChunk = 4096;
__global__ void k_seq_sum(const double *part, long n, double *out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double s = 0.0;
        for (long t = 0; t < n; ++t) s += part[t];
        *out = s;
    }
}
__global__ void k_chunk_sum_flat(const double *a, long n, double *part) {
    long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long c0 = c * kChunk;
    if (c0 >= n) return;
    long c1 = min(n, c0 + kChunk);
    double s = 0.0;
    for (long t = c0; t < c1; ++t) s += a[t];
    part[c] = s;
}

struct MgBC {
    int per[3];         // periodic axes
    int E[3];           // core upper index (xEnd) at this level
    int dirichlet;      // Dirichlet check (TEST_POISSON)
    int zeroBC;         // homogeneous Dirichlet (levels > 0)
    int tgtPads;        // residual pads: 0 = reference (z ghost 0, non-periodic 0), 1 = mirror/periodic
    int planar;         // 2D: one y point, y never periodic (poisson_d2.cc)
};

struct MgK {            // level stencil constants
    double cx, cy, cz, c7, den;
    double iden;       // RN(1 / den), for div_rn
    double lx, ly, lz;
    float fcx, fcy, fcz, fc7, fden, flx, fly, flz;
    // stretched meshes (var != 0, reference mode): the level's metric arrays
    // (poisson.cc:463-495) and spacings, read at each point
    const double *xix2, *xixx, *ety2, *etyy, *ztz2, *ztzz;
    double hx, hy, hz, hxhy, hyhz, hzhx, hxhyhz, ihx2, ihy2, ihz2, i2hx, i2hy, i2hz;
    double hx2, hz2;   // 2D (poisson.cc:406-409, 426-428)
    int var;
    int planar;        // 2D: the x-z stencils of poisson_d2.cc (with var set, metrics from the arrays)
};

static MgK make_k(const Level &L) {
    MgK k;
    k.cx = L.cx; k.cy = L.cy; k.cz = L.cz; k.c7 = L.c7; k.den = L.den;
    k.iden = 1.0 / L.den;
    k.lx = L.lx; k.ly = L.ly; k.lz = L.lz;
    k.fcx = (float)L.cx; k.fcy = (float)L.cy; k.fcz = (float)L.cz; k.fc7 = (float)L.c7; k.fden = (float)L.den;
    k.flx = (float)L.lx; k.fly = (float)L.ly; k.flz = (float)L.lz;
    k.xix2 = L.xix2; k.xixx = L.xixx; k.ety2 = L.ety2; k.etyy = L.etyy; k.ztz2 = L.ztz2; k.ztzz = L.ztzz;
    k.hx = L.hx; k.hy = L.hy; k.hz = L.hz; k.hxhy = L.hxhy; k.hyhz = L.hyhz; k.hzhx = L.hzhx; k.hxhyhz = L.hxhyhz;
    k.ihx2 = L.ihx2; k.ihy2 = L.ihy2; k.ihz2 = L.ihz2;
    k.i2hx = 1.0 / (2.0 * L.hx); k.i2hy = 1.0 / (2.0 * L.hy); k.i2hz = 1.0 / (2.0 * L.hz);   // exact: powers of two
    k.hx2 = L.hx2; k.hz2 = L.hz2;
    k.var = L.xix2 != nullptr;
    k.planar = L.planar;
    return k;
}

template <typename T> struct KSel;
template <> struct KSel<double> {
    static __device__ __forceinline__ double cx(const MgK &k) { return k.cx; }
    static __device__ __forceinline__ double cy(const MgK &k) { return k.cy; }
    static __device__ __forceinline__ double cz(const MgK &k) { return k.cz; }
    static __device__ __forceinline__ double c7(const MgK &k) { return k.c7; }
    static __device__ __forceinline__ double den(const MgK &k) { return k.den; }
    static __device__ __forceinline__ double lx(const MgK &k) { return k.lx; }
    static __device__ __forceinline__ double ly(const MgK &k) { return k.ly; }
    static __device__ __forceinline__ double lz(const MgK &k) { return k.lz; }
};
template <> struct KSel<float> {
    static __device__ __forceinline__ float cx(const MgK &k) { return k.fcx; }
    static __device__ __forceinline__ float cy(const MgK &k) { return k.fcy; }
    static __device__ __forceinline__ float cz(const MgK &k) { return k.fcz; }
    static __device__ __forceinline__ float c7(const MgK &k) { return k.fc7; }
    static __device__ __forceinline__ float den(const MgK &k) { return k.fden; }
    static __device__ __forceinline__ float lx(const MgK &k) { return k.flx; }
    static __device__ __forceinline__ float ly(const MgK &k) { return k.fly; }
    static __device__ __forceinline__ float lz(const MgK &k) { return k.flz; }
};

// Smoother update, the expression of poisson_d3.cc:156-163 at point (x, y, z).
// Uniform grid: the xixx, etyy, ztzz terms are exactly zero and omitted, the
// metric products are level constants.  Stretched mesh (FP64 only): every
// term, the metrics read at the point.
template <typename T>
__device__ __forceinline__ T mg_update(T E, T W, T N, T S, T U, T D, T r, const MgK &k, int x, int y, int z) {
    using K = KSel<T>;
    if constexpr (sizeof(T) == 8) {
        if (k.planar)   // poisson_d2.cc:126-131
            return (k.hz2 * k.xix2[x] * (E + W) * 2.0 + k.hz2 * k.xixx[x] * (E - W) * k.hx + k.hx2 * k.ztz2[z] * (U + D) * 2.0 +
                    k.hx2 * k.ztzz[z] * (U - D) * k.hz - 2.0 * k.hzhx * r) /
                   (4.0 * (k.hz2 * k.xix2[x] + k.hx2 * k.ztz2[z]));
        if (k.var)
            return (k.hyhz * k.xix2[x] * (E + W) * 2.0 + k.hyhz * k.xixx[x] * (E - W) * k.hx + k.hzhx * k.ety2[y] * (N + S) * 2.0 +
                    k.hzhx * k.etyy[y] * (N - S) * k.hy + k.hxhy * k.ztz2[z] * (U + D) * 2.0 + k.hxhy * k.ztzz[z] * (U - D) * k.hz -
                    2.0 * k.hxhyhz * r) /
                   (4.0 * (k.hyhz * k.xix2[x] + k.hzhx * k.ety2[y] + k.hxhy * k.ztz2[z]));
    }
    const T num = (K::cx(k) * (E + W)) * (T)2.0 + (K::cy(k) * (N + S)) * (T)2.0 + (K::cz(k) * (U + D)) * (T)2.0 - K::c7(k) * r;
    if constexpr (sizeof(T) == 8) return div_rn(num, k.den, k.iden);
    return num / K::den(k);
}
// Laplacian, the expression of poisson_d3.cc:99-105 at point (x, y, z); the
// divisions by (hx*hx) and (2*hx) are multiplications by exact reciprocals.
template <typename T>
__device__ __forceinline__ T mg_lap(T E, T W, T N, T S, T U, T D, T C, const MgK &k, int x, int y, int z) {
    using K = KSel<T>;
    if constexpr (sizeof(T) == 8) {
        if (k.planar)   // poisson_d2.cc:97-100
            return k.xix2[x] * (E - 2.0 * C + W) * k.ihx2 + k.xixx[x] * (E - W) * k.i2hx + k.ztz2[z] * (U - 2.0 * C + D) * k.ihz2 +
                   k.ztzz[z] * (U - D) * k.i2hz;
        if (k.var)
            return k.xix2[x] * (E - 2.0 * C + W) * k.ihx2 + k.xixx[x] * (E - W) * k.i2hx + k.ety2[y] * (N - 2.0 * C + S) * k.ihy2 +
                   k.etyy[y] * (N - S) * k.i2hy + k.ztz2[z] * (U - 2.0 * C + D) * k.ihz2 + k.ztzz[z] * (U - D) * k.i2hz;
    }
    return K::lx(k) * (E - (T)2.0 * C + W) + K::ly(k) * (N - (T)2.0 * C + S) + K::lz(k) * (U - (T)2.0 * C + D);
}

__device__ __forceinline__ bool core_pt(const int E[3], int &i, int &j, int &k) {
    k = blockIdx.x * blockDim.x + threadIdx.x;
    j = blockIdx.y * blockDim.y + threadIdx.y;
    i = blockIdx.z * blockDim.z + threadIdx.z;
    return i <= E[0] && j <= E[1] && k <= E[2];
}

// Write v at (i,j,k) and at every face-ghost position whose imposeBC image is
// (i,j,k): periodic -1 <- E-1, E+1 <- 1; Neumann -1 <- 1, E+1 <- E-1;
// homogeneous Dirichlet the negated mirror (TEST_POISSON, levels > 0).
template <typename T>
__device__ __forceinline__ void put_scatter(const View3<T> &P, int i, int j, int k, T v, const MgBC &bc) {
    P(i, j, k) = v;
    int q[3] = {i, j, k};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int E = bc.E[d];
        bool dirich = bc.dirichlet && !bc.per[d];
        if (dirich && !bc.zeroBC) continue;   // fixed wall values are set once per solve
        T s = (dirich && bc.zeroBC) ? (T)(-1.0) : (T)1.0;
        int g[2] = {-2, -2};
        if (bc.per[d]) { if (q[d] == E - 1) g[0] = -1; if (q[d] == 1) g[1] = E + 1; }
        else { if (q[d] == 1) g[0] = -1; if (q[d] == E - 1) g[1] = E + 1; }
        for (int t = 0; t < 2; ++t) {
            if (g[t] == -2) continue;
            int r[3] = {i, j, k};
            r[d] = g[t];
            P(r[0], r[1], r[2]) = s * v;
        }
    }
}

// One Jacobi sweep (poisson_d3.cc:153-168).  zero_guess: the incoming iterate
// is identically 0 (pressureData = 0 before smoothing a coarse level,
// poisson.cc:258).  omega = 1 reproduces the reference exactly.
template <typename T, bool ZERO>
__global__ void k_mg_sweep(View3<T> out, View3<const T> in, View3<const T> r, MgK kk, MgBC bc, T omega) {
    int i, j, k;
    if (!core_pt(bc.E, i, j, k)) return;
    T v;
    if (ZERO) {
        v = mg_update<T>((T)0, (T)0, (T)0, (T)0, (T)0, (T)0, r(i, j, k), kk, i, j, k);
        if (omega != (T)1.0) v = omega * v;
    } else {
        T C = in(i, j, k);
        v = mg_update<T>(in(i + 1, j, k), in(i - 1, j, k), in(i, j + 1, k), in(i, j - 1, k), in(i, j, k + 1), in(i, j, k - 1),
                         r(i, j, k), kk, i, j, k);
        if (omega != (T)1.0) v = C + omega * (v - C);
    }
    put_scatter(out, i, j, k, v, bc);
}

// computeResidual (poisson_d3.cc:90-111): tmp(core) = r - Lap(p).
template <typename T>
__global__ void k_mg_residual(View3<T> tmp, View3<const T> p, View3<const T> r, MgK kk, MgBC bc) {
    int i, j, k;
    if (!core_pt(bc.E, i, j, k)) return;
    T lap = mg_lap<T>(p(i + 1, j, k), p(i - 1, j, k), p(i, j + 1, k), p(i, j - 1, k), p(i, j, k + 1), p(i, j, k - 1), p(i, j, k), kk, i, j, k);
    tmp(i, j, k) = r(i, j, k) - lap;
}

// Value of the residual array at a possibly-ghost index after updatePads
// (reference pads: x/y periodic copies of whole planes, everything else 0;
// the z ghosts stay 0 even for periodic z), or after a mirror/periodic fill
// in the target modes.
template <typename T>
__device__ __forceinline__ T pad_val(const View3<const T> &t, int i, int j, int k, const MgBC &bc) {
    int q[3] = {i, j, k};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int E = bc.E[d];
        if (q[d] >= 0 && q[d] <= E) continue;
        if (bc.tgtPads) {
            if (bc.per[d]) q[d] = q[d] < 0 ? E - 1 : 1;
            else q[d] = q[d] < 0 ? 1 : E - 1;
        } else {
            if (d == 2 || !bc.per[d]) return (T)0;
            q[d] = q[d] < 0 ? E - 1 : 1;
        }
    }
    return t(q[0], q[1], q[2]);
}

// coarsen (poisson_d3.cc:250-298): 27-point full weighting in the reference's
// summation order.  bcf describes the fine level, Ec the coarse core.
template <typename T>
__global__ void k_mg_restrict(View3<T> rc, View3<const T> t, MgBC bcf, MgBC bcc) {
    int i, j, k;
    if (!core_pt(bcc.E, i, j, k)) return;
    int i2 = 2 * i, j2 = 2 * j, k2 = 2 * k;
    if (bcf.planar) {   // poisson_d2.cc:207-225: 9-point full weighting in the y = 0 plane
        const bool in2 = i2 > 0 && k2 > 0 && i2 < bcf.E[0] && k2 < bcf.E[2];
        auto Q = [&](int a, int c) -> T { return in2 ? t(a, 0, c) : pad_val(t, a, 0, c, bcf); };
        T facePoints = (Q(i2 + 1, k2) + Q(i2 - 1, k2) + Q(i2, k2 + 1) + Q(i2, k2 - 1)) * (T)0.125;
        T vertPoints = (Q(i2 + 1, k2 + 1) + Q(i2 + 1, k2 - 1) + Q(i2 - 1, k2 + 1) + Q(i2 - 1, k2 - 1)) * (T)0.0625;
        rc(i, 0, k) = facePoints + vertPoints + t(i2, 0, k2) * (T)0.25;
        return;
    }
    bool interior = i2 > 0 && j2 > 0 && k2 > 0 && i2 < bcf.E[0] && j2 < bcf.E[1] && k2 < bcf.E[2];
    auto T_ = [&](int a, int b, int c) -> T { return interior ? t(a, b, c) : pad_val(t, a, b, c, bcf); };
    T facePoints = (T_(i2 + 1, j2, k2) + T_(i2 - 1, j2, k2) + T_(i2, j2 + 1, k2) + T_(i2, j2 - 1, k2) +
                    T_(i2, j2, k2 + 1) + T_(i2, j2, k2 - 1)) * (T)0.0625;
    T edgePoints = (T_(i2 + 1, j2 + 1, k2) + T_(i2 + 1, j2 - 1, k2) + T_(i2 - 1, j2 - 1, k2) + T_(i2 - 1, j2 + 1, k2) +
                    T_(i2, j2 + 1, k2 + 1) + T_(i2, j2 - 1, k2 + 1) + T_(i2, j2 - 1, k2 - 1) + T_(i2, j2 + 1, k2 - 1) +
                    T_(i2 + 1, j2, k2 + 1) + T_(i2 + 1, j2, k2 - 1) + T_(i2 - 1, j2, k2 - 1) + T_(i2 - 1, j2, k2 + 1)) * (T)0.03125;
    T vertPoints = (T_(i2 + 1, j2 + 1, k2 + 1) + T_(i2 + 1, j2 + 1, k2 - 1) + T_(i2 + 1, j2 - 1, k2 + 1) +
                    T_(i2 - 1, j2 + 1, k2 + 1) + T_(i2 + 1, j2 - 1, k2 - 1) + T_(i2 - 1, j2 + 1, k2 - 1) +
                    T_(i2 - 1, j2 - 1, k2 + 1) + T_(i2 - 1, j2 - 1, k2 - 1)) * (T)0.015625;
    rc(i, j, k) = facePoints + edgePoints + vertPoints + t(i2, j2, k2) * (T)0.125;
}

// prolong (poisson_d3.cc:301-388) followed by pressureData += smoothedPres
// (poisson.cc:271); the saved data is the fine array itself, updated in place.
template <typename T>
__global__ void k_mg_prolong_add(View3<T> pf, View3<const T> pc, MgBC bc, int add) {
    int i, j, k;
    if (!core_pt(bc.E, i, j, k)) return;
    int i2 = i / 2, j2 = j / 2, k2 = k / 2;
    bool io = i & 1, jo = j & 1, ko = k & 1;
    T v;
    const View3<const T> &C = pc;
    if (io) {
        if (jo) {
            if (ko) v = (C(i2, j2, k2) + C(i2 + 1, j2, k2) + C(i2, j2 + 1, k2) + C(i2, j2, k2 + 1) + C(i2 + 1, j2 + 1, k2) +
                         C(i2 + 1, j2, k2 + 1) + C(i2, j2 + 1, k2 + 1) + C(i2 + 1, j2 + 1, k2 + 1)) * (T)0.125;
            else v = (C(i2, j2, k2) + C(i2, j2 + 1, k2) + C(i2 + 1, j2, k2) + C(i2 + 1, j2 + 1, k2)) * (T)0.25;
        } else {
            if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1) + C(i2 + 1, j2, k2) + C(i2 + 1, j2, k2 + 1)) * (T)0.25;
            else v = (C(i2, j2, k2) + C(i2 + 1, j2, k2)) * (T)0.5;
        }
    } else {
        if (jo) {
            if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1) + C(i2, j2 + 1, k2) + C(i2, j2 + 1, k2 + 1)) * (T)0.25;
            else v = (C(i2, j2, k2) + C(i2, j2 + 1, k2)) * (T)0.5;
        } else {
            if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1)) * (T)0.5;
            else v = C(i2, j2, k2);
        }
    }
    if (add) v = v + pf(i, j, k);
    put_scatter(pf, i, j, k, v, bc);
}

// Coarsest level (poisson_d3.cc:190-247): lexicographic Gauss-Seidel, run as a
// hyperplane wavefront (points with equal i+j+k are independent, and visiting
// the planes in increasing order gives every point exactly the lexicographic
// mix of updated and old neighbours).  Ghosts are refreshed before each sweep
// (imposeBC) and read from the pre-sweep state, as in the reference.  The
// iteration loop runs on the device; it stops below tol or after maxCount+1
// sweeps.  tgtMode: subtract the trapezoidal mean of r first and stop on a
// relative reduction instead.
template <typename T>
__device__ void smem_impose_bc(T *p, int X, int Y, int Z, const MgBC &bc, const T *wx, const T *wy, const T *wz) {
    int sy = Z + 3, sx = (Y + 3) * (Z + 3);
    auto at = [&](int i, int j, int k) -> T & { return p[(i + 1) * sx + (j + 1) * sy + (k + 1)]; };
    int tid = threadIdx.x, nt = blockDim.x;
    // updatePads: periodic x planes then y planes (full extents)
    if (bc.per[0]) {
        for (int t = tid; t < (Y + 3) * (Z + 3); t += nt) { int j = t / (Z + 3) - 1, k = t % (Z + 3) - 1; at(X + 1, j, k) = at(1, j, k); at(-1, j, k) = at(X - 1, j, k); }
        __syncthreads();
    }
    if (bc.per[1]) {
        for (int t = tid; t < (X + 3) * (Z + 3); t += nt) { int i = t / (Z + 3) - 1, k = t % (Z + 3) - 1; at(i, Y + 1, k) = at(i, 1, k); at(i, -1, k) = at(i, Y - 1, k); }
        __syncthreads();
    }
    if (!bc.per[0]) {
        for (int t = tid; t < (Y + 3) * (Z + 3); t += nt) {
            int j = t / (Z + 3) - 1, k = t % (Z + 3) - 1;
            if (bc.dirichlet) {
                if (bc.zeroBC) { at(-1, j, k) = -at(1, j, k); at(X + 1, j, k) = -at(X - 1, j, k); }
                else { T w = wx[(j + 1) * (Z + 3) + (k + 1)]; at(-1, j, k) = w; at(X + 1, j, k) = w; }
            } else { at(-1, j, k) = at(1, j, k); at(X + 1, j, k) = at(X - 1, j, k); }
        }
        __syncthreads();
    }
    if (!bc.per[1]) {
        for (int t = tid; t < (X + 3) * (Z + 3); t += nt) {
            int i = t / (Z + 3) - 1, k = t % (Z + 3) - 1;
            if (bc.dirichlet) {
                if (bc.zeroBC) { at(i, -1, k) = -at(i, 1, k); at(i, Y + 1, k) = -at(i, Y - 1, k); }
                else { T w = wy[(i + 1) * (Z + 3) + (k + 1)]; at(i, -1, k) = w; at(i, Y + 1, k) = w; }
            } else { at(i, -1, k) = at(i, 1, k); at(i, Y + 1, k) = at(i, Y - 1, k); }
        }
        __syncthreads();
    }
    for (int t = tid; t < (X + 3) * (Y + 3); t += nt) {
        int i = t / (Y + 3) - 1, j = t % (Y + 3) - 1;
        if (bc.per[2]) { at(i, j, -1) = at(i, j, Z - 1); at(i, j, Z + 1) = at(i, j, 1); }
        else if (bc.dirichlet) {
            if (bc.zeroBC) { at(i, j, -1) = -at(i, j, 1); at(i, j, Z + 1) = -at(i, j, Z - 1); }
            else { T w = wz[(i + 1) * (Y + 3) + (j + 1)]; at(i, j, -1) = w; at(i, j, Z + 1) = w; }
        } else { at(i, j, -1) = at(i, j, 1); at(i, j, Z + 1) = at(i, j, Z - 1); }
    }
    __syncthreads();
}

// The coarsest-level solve on shared-memory arrays: p (zeroed by the caller)
// and r in the padded layout of a level with core 0..X, 0..Y, 0..Z.
template <typename T>
__device__ void coarse_gs(T *p, T *r, int X, int Y, int Z, const MgK &kk, const MgBC &bc, T tol, int maxCount, int tgtMode,
                          long long *iters) {
    __shared__ T red[32];
    __shared__ int stop;
    int sy = Z + 3, sx = (Y + 3) * (Z + 3);
    auto at = [&](T *a, int i, int j, int k) -> T & { return a[(i + 1) * sx + (j + 1) * sy + (k + 1)]; };
    int tid = threadIdx.x, nt = blockDim.x;
    T thresh = tol;
    if (tgtMode) {
        // trapezoidal-weight mean of r over the core (weights 1/2 on end planes)
        T s = 0, w = 0;
        for (int t = tid; t < (X + 1) * (Y + 1) * (Z + 1); t += nt) {
            int k = t % (Z + 1), j = (t / (Z + 1)) % (Y + 1), i = t / ((Z + 1) * (Y + 1));
            T wt = (T)((i == 0 || i == X) ? 0.5 : 1.0) * (T)((j == 0 || j == Y) ? 0.5 : 1.0) * (T)((k == 0 || k == Z) ? 0.5 : 1.0);
            s += wt * at(r, i, j, k); w += wt;
        }
        s = warp_sum(s); w = warp_sum(w);
        __shared__ T ss[32], sw[32];
        if ((tid & 31) == 0) { ss[tid >> 5] = s; sw[tid >> 5] = w; }
        __syncthreads();
        if (tid == 0) { T S = 0, W = 0; for (int q = 0; q < nt / 32; ++q) { S += ss[q]; W += sw[q]; } ss[0] = S / W; }
        __syncthreads();
        T mean = ss[0];
        T m = 0;
        for (int t = tid; t < (X + 1) * (Y + 1) * (Z + 1); t += nt) {
            int k = t % (Z + 1), j = (t / (Z + 1)) % (Y + 1), i = t / ((Z + 1) * (Y + 1));
            at(r, i, j, k) -= mean;
            m = fmax(m, fabs(at(r, i, j, k)));
        }
        m = warp_max(m);
        if ((tid & 31) == 0) red[tid >> 5] = m;
        __syncthreads();
        if (tid == 0) { T M = 0; for (int q = 0; q < nt / 32; ++q) M = fmax(M, red[q]); red[0] = M; }
        __syncthreads();
        thresh = tol * red[0];
        __syncthreads();
    }
    int iterCount = 0;
    long long sweeps = 0;
    int smax = X + Y + Z;
    while (true) {
        smem_impose_bc(p, X, Y, Z, bc, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr);
        for (int s = 0; s <= smax; ++s) {
            for (int t = tid; t < (X + 1) * (Y + 1); t += nt) {
                int i = t / (Y + 1), j = t % (Y + 1);
                int k = s - i - j;
                if (k < 0 || k > Z) continue;
                at(p, i, j, k) = mg_update<T>(at(p, i + 1, j, k), at(p, i - 1, j, k), at(p, i, j + 1, k), at(p, i, j - 1, k),
                                              at(p, i, j, k + 1), at(p, i, j, k - 1), at(r, i, j, k), kk, i, j, k);
            }
            __syncthreads();
        }
        sweeps += 1;
        T localMax = (T)-1.0e-10;
        for (int t = tid; t < (X + 1) * (Y + 1) * (Z + 1); t += nt) {
            int k = t % (Z + 1), j = (t / (Z + 1)) % (Y + 1), i = t / ((Z + 1) * (Y + 1));
            T lap = mg_lap<T>(at(p, i + 1, j, k), at(p, i - 1, j, k), at(p, i, j + 1, k), at(p, i, j - 1, k), at(p, i, j, k + 1),
                              at(p, i, j, k - 1), at(p, i, j, k), kk, i, j, k);
            T v = fabs(at(r, i, j, k) - lap);
            if (v != v) v = (T)INFINITY;
            if (v > localMax) localMax = v;
        }
        localMax = warp_max(localMax);
        if ((tid & 31) == 0) red[tid >> 5] = localMax;
        __syncthreads();
        if (tid == 0) {
            T M = red[0];
            for (int q = 1; q < nt / 32; ++q) M = fmax(M, red[q]);
            int st = 0;
            if (M < thresh) st = 1;
            else {
                iterCount += 1;
                if (iterCount > maxCount) st = 1;
            }
            stop = st;
        }
        __syncthreads();
        if (stop) break;
    }
    smem_impose_bc(p, X, Y, Z, bc, (const T *)nullptr, (const T *)nullptr, (const T *)nullptr);
    __syncthreads();
    if (tid == 0 && iters) *iters += sweeps;
}

// The target modes' coarsest solve inside k_mg_tail, by one warp: the
// compatible right-hand side (trapezoidal mean removed), then red-black
// Gauss-Seidel sweeps (the two colours of i+j+k, ghosts refreshed before each)
// until max|r - Lp| falls below tol times its initial value or maxCount
// sweeps.  A warp needs no block barriers, which bound the block-wide
// wavefront sweep on a level of about a hundred points.  Only the two
// colours' order differs from the lexicographic sweep; the target modes only
// need a small coarse residual, not the reference's iterates.
template <typename T>
__device__ void warp_ghosts(T *p, int X, int Y, int Z, const MgBC &bc) {
    int lane = threadIdx.x & 31, sy = Z + 3, sx = (Y + 3) * sy;
    auto at = [&](int i, int j, int k) -> T & { return p[(i + 1) * sx + (j + 1) * sy + (k + 1)]; };
    for (int t = lane; t < (Y + 3) * (Z + 3); t += 32) {
        int j = t / (Z + 3) - 1, k = t % (Z + 3) - 1;
        if (bc.per[0]) { at(X + 1, j, k) = at(1, j, k); at(-1, j, k) = at(X - 1, j, k); }
        else { at(-1, j, k) = at(1, j, k); at(X + 1, j, k) = at(X - 1, j, k); }
    }
    __syncwarp();
    for (int t = lane; t < (X + 3) * (Z + 3); t += 32) {
        int i = t / (Z + 3) - 1, k = t % (Z + 3) - 1;
        if (bc.per[1]) { at(i, Y + 1, k) = at(i, 1, k); at(i, -1, k) = at(i, Y - 1, k); }
        else { at(i, -1, k) = at(i, 1, k); at(i, Y + 1, k) = at(i, Y - 1, k); }
    }
    __syncwarp();
    for (int t = lane; t < (X + 3) * (Y + 3); t += 32) {
        int i = t / (Y + 3) - 1, j = t % (Y + 3) - 1;
        if (bc.per[2]) { at(i, j, -1) = at(i, j, Z - 1); at(i, j, Z + 1) = at(i, j, 1); }
        else { at(i, j, -1) = at(i, j, 1); at(i, j, Z + 1) = at(i, j, Z - 1); }
    }
    __syncwarp();
}

template <typename T>
__device__ void coarse_rbgs_warp(T *p, T *r, int X, int Y, int Z, const MgK &kk, const MgBC &bc, T tol, int maxCount, long long *iters) {
    int lane = threadIdx.x & 31, sy = Z + 3, sx = (Y + 3) * sy;
    int n = (X + 1) * (Y + 1) * (Z + 1);
    auto at = [&](T *a, int i, int j, int k) -> T & { return a[(i + 1) * sx + (j + 1) * sy + (k + 1)]; };
    T sm = 0, sw = 0;
    for (int t = lane; t < n; t += 32) {
        int k = t % (Z + 1), j = (t / (Z + 1)) % (Y + 1), i = t / ((Z + 1) * (Y + 1));
        T wt = (T)((i == 0 || i == X) ? 0.5 : 1.0) * (T)((j == 0 || j == Y) ? 0.5 : 1.0) * (T)((k == 0 || k == Z) ? 0.5 : 1.0);
        sm += wt * at(r, i, j, k);
        sw += wt;
    }
    T mean = warp_sum(sm) / warp_sum(sw);
    T m0 = 0;
    for (int t = lane; t < n; t += 32) {
        int k = t % (Z + 1), j = (t / (Z + 1)) % (Y + 1), i = t / ((Z + 1) * (Y + 1));
        at(r, i, j, k) -= mean;
        m0 = fmax(m0, fabs(at(r, i, j, k)));
    }
    __syncwarp();
    T thresh = tol * warp_max(m0);
    long long sweeps = 0;
    for (int it = 0; it <= maxCount; ++it) {
        for (int colour = 0; colour < 2; ++colour) {
            warp_ghosts(p, X, Y, Z, bc);
            for (int t = lane; t < n; t += 32) {
                int k = t % (Z + 1), j = (t / (Z + 1)) % (Y + 1), i = t / ((Z + 1) * (Y + 1));
                if (((i + j + k) & 1) != colour) continue;
                at(p, i, j, k) = mg_update<T>(at(p, i + 1, j, k), at(p, i - 1, j, k), at(p, i, j + 1, k), at(p, i, j - 1, k),
                                              at(p, i, j, k + 1), at(p, i, j, k - 1), at(r, i, j, k), kk, i, j, k);
            }
            __syncwarp();
        }
        sweeps += 1;
        warp_ghosts(p, X, Y, Z, bc);
        T m = 0;
        for (int t = lane; t < n; t += 32) {
            int k = t % (Z + 1), j = (t / (Z + 1)) % (Y + 1), i = t / ((Z + 1) * (Y + 1));
            T lap = mg_lap<T>(at(p, i + 1, j, k), at(p, i - 1, j, k), at(p, i, j + 1, k), at(p, i, j - 1, k), at(p, i, j, k + 1),
                              at(p, i, j, k - 1), at(p, i, j, k), kk, i, j, k);
            T v = fabs(at(r, i, j, k) - lap);
            if (v != v) v = (T)INFINITY;
            m = fmax(m, v);
        }
        if (warp_max(m) < thresh) break;
    }
    if (lane == 0 && iters) *iters += sweeps;
}

template <typename T>
__global__ void k_mg_coarse(View3<T> pg, View3<const T> rg, MgK kk, MgBC bc, T tol, int maxCount, int tgtMode,
                            long long *iters) {
    extern __shared__ unsigned char smraw[];
    int X = bc.E[0], Y = bc.E[1], Z = bc.E[2];
    int n = (X + 3) * (Y + 3) * (Z + 3);
    T *p = reinterpret_cast<T *>(smraw);
    T *r = p + n;
    for (int t = threadIdx.x; t < n; t += blockDim.x) { p[t] = (T)0; r[t] = rg.p[t]; }   // pressureData(d) = 0 (poisson.cc:258)
    __syncthreads();
    coarse_gs(p, r, X, Y, Z, kk, bc, tol, maxCount, tgtMode, iters);
    for (int t = threadIdx.x; t < n; t += blockDim.x) pg.p[t] = p[t];
}

// ------------------------------------------------------------------ Gauss-Seidel smoothing
// gsSmooth = 1 (poisson_d3.cc:137-150): every level is smoothed in place in
// lexicographic order, so each point sees the updated values of its (i-1),
// (j-1), (k-1) neighbours and the old values of its (i+1), (j+1), (k+1)
// neighbours.  The points of one hyperplane i + j + k = s depend only on
// plane s - 1 (updated) and plane s + 1 (old): updating the planes in
// increasing s, each plane in parallel, performs the same arithmetic on the
// same operands as the lexicographic loop, bit for bit, in X + Y + Z + 1
// dependent stages.  imposeBC runs before every sweep and once after
// (poisson_d3.cc:124, 181); the ghosts a sweep reads are those of the state
// before it, which the stages never write.

// Levels whose iterate and right-hand side fit in shared memory (at most
// kGsBlockSmem bytes together): one CTA, the stages separated by
// __syncthreads.  zero: pressureData = 0 on entry.
constexpr size_t kGsBlockSmem = 200 * 1024;
__global__ void k_mg_gs_block(View3<double> pg, View3<const double> rg, MgK kk, MgBC bc, int count, int zero,
                              const double *wx, const double *wy, const double *wz) {
    extern __shared__ unsigned char smraw[];
    const int X = bc.E[0], Y = bc.E[1], Z = bc.E[2];
    const int n = (X + 3) * (Y + 3) * (Z + 3), sy = Z + 3, sx = (Y + 3) * (Z + 3);
    double *p = reinterpret_cast<double *>(smraw);
    double *r = p + n;
    auto at = [&](double *a, int i, int j, int k) -> double & { return a[(i + 1) * sx + (j + 1) * sy + (k + 1)]; };
    for (int t = threadIdx.x; t < n; t += blockDim.x) { p[t] = zero ? 0.0 : pg.p[t]; r[t] = rg.p[t]; }
    __syncthreads();
    for (int it = 0; it < count; ++it) {
        smem_impose_bc(p, X, Y, Z, bc, wx, wy, wz);
        for (int s = 0; s <= X + Y + Z; ++s) {
            for (int t = threadIdx.x; t < (X + 1) * (Y + 1); t += blockDim.x) {
                int i = t / (Y + 1), j = t % (Y + 1), k = s - i - j;
                if (k < 0 || k > Z) continue;
                at(p, i, j, k) = mg_update<double>(at(p, i + 1, j, k), at(p, i - 1, j, k), at(p, i, j + 1, k), at(p, i, j - 1, k),
                                                   at(p, i, j, k + 1), at(p, i, j, k - 1), at(r, i, j, k), kk, i, j, k);
            }
            __syncthreads();
        }
    }
    smem_impose_bc(p, X, Y, Z, bc, wx, wy, wz);
    for (int t = threadIdx.x; t < n; t += blockDim.x) pg.p[t] = p[t];
}

// Value that imposeBC (x planes, y planes, then z planes over full extents,
// poisson_d3.cc:575-668 with updatePads first) leaves at the ghost point
// (i, j, k), resolved from the core: the last writer first (z, then y, then
// x); periodic and mirror copies map one coordinate to its image, Dirichlet
// walls of the check case end the chain with their fixed value, and
// homogeneous Dirichlet images change sign.
__device__ __forceinline__ double mg_ghost_value(const View3<const double> &p, int i, int j, int k, const MgBC &bc,
                                                 const double *wx, const double *wy, const double *wz) {
    int q[3] = {i, j, k};
    const int E1 = bc.E[1], E2 = bc.E[2];
    double sign = 1.0;
    for (int d = 2; d >= 0; --d) {
        int E = bc.E[d];
        if (q[d] >= 0 && q[d] <= E) continue;
        if (bc.per[d]) { q[d] = q[d] < 0 ? E - 1 : 1; continue; }
        if (bc.dirichlet && !bc.zeroBC) {
            const double *w = d == 0 ? wx : d == 1 ? wy : wz;
            int a = d == 0 ? q[1] : q[0], b = d == 2 ? q[1] : q[2];
            int nb = d == 2 ? (E1 + 3) : (E2 + 3);
            return sign * w[(a + 1) * nb + (b + 1)];
        }
        if (bc.dirichlet) sign = -sign;
        q[d] = q[d] < 0 ? 1 : E - 1;
    }
    return sign * __ldcg(&p(q[0], q[1], q[2]));
}

// Grid-wide barrier for the cooperative Gauss-Seidel kernel: block arrivals
// are counted on *count (zeroed before the launch); the b-th barrier waits
// for b * gridDim.x arrivals.  The wait is bounded: after kGsSpinLimit polls
// (about a second) the block records the failure in *err and every block
// leaves the kernel at its next barrier.
constexpr long long kGsSpinLimit = 1ll << 24;
__device__ __forceinline__ bool gs_grid_sync(unsigned *count, unsigned target, int *err) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(count, 1u);
        long long spins = 0;
        int good = 1;
        while (*(volatile unsigned *)count < target) {
            if (*(volatile int *)err) { good = 0; break; }
            if (++spins > kGsSpinLimit) { atomicExch(err, 1); good = 0; break; }
            __nanosleep(64);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Levels too large for one CTA's shared memory: a cooperative launch over
// gridDim.x co-resident blocks, the stages separated by grid barriers.  The
// iterate is read past L1 (ld.global.cg), so a block never sees a line that
// another block has updated since.  `count` sweeps, each preceded by the
// ghost fill, and a final ghost fill.
__global__ void __launch_bounds__(256) k_mg_gs_grid(View3<double> p, View3<const double> r, MgK kk, MgBC bc, int count,
                                                    unsigned *sync, int *err, const double *wx, const double *wy,
                                                    const double *wz) {
    const int X = bc.E[0], Y = bc.E[1], Z = bc.E[2];
    const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x, nt = (long)gridDim.x * blockDim.x;
    const View3<const double> pc{p.p, {p.n[0], p.n[1], p.n[2]}, p.sx, p.sy};
    // ghost points: two full x planes, two y planes (x core), two z planes (x, y core)
    const long fx = (long)(Y + 3) * (Z + 3), fy = (long)(X + 1) * (Z + 3), fz = (long)(X + 1) * (Y + 1);
    const long ng = 2 * (fx + fy + fz);
    unsigned target = 0;
    for (int it = 0;; ++it) {
        for (long t = tid; t < ng; t += nt) {
            int i, j, k;
            long u = t;
            if (u < 2 * fx) { i = u < fx ? -1 : X + 1; u %= fx; j = (int)(u / (Z + 3)) - 1; k = (int)(u % (Z + 3)) - 1; }
            else if ((u -= 2 * fx) < 2 * fy) { j = u < fy ? -1 : Y + 1; u %= fy; i = (int)(u / (Z + 3)); k = (int)(u % (Z + 3)) - 1; }
            else { u -= 2 * fy; k = u < fz ? -1 : Z + 1; u %= fz; i = (int)(u / (Y + 1)); j = (int)(u % (Y + 1)); }
            p(i, j, k) = mg_ghost_value(pc, i, j, k, bc, wx, wy, wz);   // reads the core past L1
        }
        if (it == count) break;
        target += gridDim.x;
        if (!gs_grid_sync(sync, target, err)) return;
        for (int s = 0; s <= X + Y + Z; ++s) {
            const int ilo = max(0, s - Y - Z), ihi = min(X, s), jlo = max(0, s - X - Z), jhi = min(Y, s);
            const long nj = jhi - jlo + 1, m = (long)(ihi - ilo + 1) * nj;
            for (long t = tid; t < m; t += nt) {
                const int i = ilo + (int)(t / nj), j = jlo + (int)(t % nj), k = s - i - j;
                if (k < 0 || k > Z) continue;
                p(i, j, k) = mg_update<double>(__ldcg(&p(i + 1, j, k)), __ldcg(&p(i - 1, j, k)), __ldcg(&p(i, j + 1, k)),
                                               __ldcg(&p(i, j - 1, k)), __ldcg(&p(i, j, k + 1)), __ldcg(&p(i, j, k - 1)), r(i, j, k), kk, i, j, k);
            }
            target += gridDim.x;
            if (!gs_grid_sync(sync, target, err)) return;
        }
    }
}

// ------------------------------------------------------------------ FP64 drivers
// Load the level-0 right-hand side: residualData(0)(core) = rhs(core), then
// updatePads (poisson.cc:114-118); per-block partial sums for the padded mean.
__global__ void k_mg_load(View3<double> r0, View3<const double> rhs, MgBC bc, double *part) {
    __shared__ double sm[32];
    long n = r0.size();
    double s = 0;
    int E1 = bc.E[1], E2 = bc.E[2];
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        int k = (int)(t % (E2 + 3)) - 1;
        int j = (int)((t / (E2 + 3)) % (E1 + 3)) - 1;
        int i = (int)(t / ((long)(E2 + 3) * (E1 + 3))) - 1;
        int q[3] = {i, j, k};
        bool zero = false;
        // z ghosts: never written by updatePads; x/y ghosts: periodic copies.
        if (k < 0 || k > E2) zero = true;
        for (int d = 0; d < 2 && !zero; ++d) {
            int E = bc.E[d];
            if (q[d] >= 0 && q[d] <= E) continue;
            if (!bc.per[d]) { zero = true; break; }
            q[d] = q[d] < 0 ? E - 1 : 1;
        }
        double v = zero ? 0.0 : rhs(q[0], q[1], q[2]);
        r0.p[t] = v;
        s += v;
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) { double S = 0; for (int w = 0; w < (int)(blockDim.x >> 5); ++w) S += sm[w]; part[blockIdx.x] = S; }
}

// residualData(0) -= mean (whole padded array, poisson.cc:128); block max of |r|.
__global__ void k_mg_sub_mean(double *r, long n, const double *sum, double count, double *maxabs) {
    double mean = (*sum / count) / 1.0;
    double m = 0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        double v = r[t] - mean;
        r[t] = v;
        m = fmax(m, fabs(v));
    }
    block_max_to(m, maxabs);
}

// pressureData(0)(core) = inFn(core) with face ghosts filled (poisson.cc:115, imposeBC).
template <typename T>
__global__ void k_mg_init_p(View3<T> p, View3<const double> src, MgBC bc) {
    int i, j, k;
    if (!core_pt(bc.E, i, j, k)) return;
    put_scatter(p, i, j, k, (T)src(i, j, k), bc);
}

// Full ghost fill of level 0 with the composition order of imposeBC (x, y, z
// planes over full extents), written to dst (the whole padded Pp array).
__global__ void k_mg_output(View3<double> dst, View3<const double> p, MgBC bc, const double *wx, const double *wy, const double *wz) {
    long n = dst.size();
    int E1 = bc.E[1], E2 = bc.E[2];
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        int k = (int)(t % (E2 + 3)) - 1;
        int j = (int)((t / (E2 + 3)) % (E1 + 3)) - 1;
        int i = (int)(t / ((long)(E2 + 3) * (E1 + 3))) - 1;
        int q[3] = {i, j, k};
        double sign = 1.0;
        double value = 0;
        bool fixed = false;
        // resolve the last writer first: z plane op, then y, then x
        for (int d = 2; d >= 0; --d) {
            int E = bc.E[d];
            if (q[d] >= 0 && q[d] <= E) continue;
            if (bc.per[d]) { q[d] = q[d] < 0 ? E - 1 : 1; continue; }
            if (bc.dirichlet && !bc.zeroBC) {
                const double *w = d == 0 ? wx : d == 1 ? wy : wz;
                int a = d == 0 ? q[1] : q[0], b = d == 2 ? q[1] : q[2];
                int nb = d == 2 ? (E1 + 3) : (E2 + 3);
                value = w[(a + 1) * nb + (b + 1)];
                fixed = true;
                break;
            }
            if (bc.dirichlet) sign = -sign;
            q[d] = q[d] < 0 ? 1 : E - 1;
        }
        dst.p[t] = fixed ? sign * value : sign * p(q[0], q[1], q[2]);
    }
}

// computeError (poisson_d3.cc:391-459) at level 0: max over the core of
// |Lap(p) - r| (norm 1) or the per-block sums of squares (norm 2).
__global__ void k_mg_error_sq(View3<const double> p, View3<const double> r, MgK kk, MgBC bc, double *partNum, double *partDen) {
    int E1 = bc.E[1], E2 = bc.E[2];
    long n = (long)(bc.E[0] + 1) * (E1 + 1) * (E2 + 1);
    long c = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long c0 = c * kChunk;
    if (c0 >= n) return;
    long c1 = min(n, c0 + kChunk);
    double sn = 0.0, sd = 0.0;
    for (long t = c0; t < c1; ++t) {
        int k = (int)(t % (E2 + 1)), j = (int)((t / (E2 + 1)) % (E1 + 1)), i = (int)(t / ((long)(E2 + 1) * (E1 + 1)));
        double lap = mg_lap<double>(p(i + 1, j, k), p(i - 1, j, k), p(i, j + 1, k), p(i, j - 1, k), p(i, j, k + 1), p(i, j, k - 1),
                                    p(i, j, k), kk, i, j, k);
        double v = fabs(lap - r(i, j, k));
        sn += v * v;
        sd += r(i, j, k) * r(i, j, k);
    }
    partNum[c] = sn;
    partDen[c] = sd;
}

__global__ void k_mg_error(View3<const double> p, View3<const double> r, MgK kk, MgBC bc, int norm, double *maxv,
                           double *partNum, double *partDen) {
    __shared__ double s1[32], s2[32];
    int E0 = bc.E[0], E1 = bc.E[1], E2 = bc.E[2];
    long n = (long)(E0 + 1) * (E1 + 1) * (E2 + 1);
    double m = 0, sn = 0, sd = 0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        int k = (int)(t % (E2 + 1)), j = (int)((t / (E2 + 1)) % (E1 + 1)), i = (int)(t / ((long)(E2 + 1) * (E1 + 1)));
        double lap = mg_lap<double>(p(i + 1, j, k), p(i - 1, j, k), p(i, j + 1, k), p(i, j - 1, k), p(i, j, k + 1), p(i, j, k - 1),
                                    p(i, j, k), kk, i, j, k);
        double v = fabs(lap - r(i, j, k));
        if (v != v) v = INFINITY;
        m = fmax(m, v);
        sn += v * v;
        sd += r(i, j, k) * r(i, j, k);
    }
    if (norm == 1) { block_max_to(m, maxv); return; }
    sn = warp_sum(sn); sd = warp_sum(sd);
    if ((threadIdx.x & 31) == 0) { s1[threadIdx.x >> 5] = sn; s2[threadIdx.x >> 5] = sd; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double A = 0, B = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { A += s1[w]; B += s2[w]; }
        partNum[blockIdx.x] = A; partDen[blockIdx.x] = B;
    }
}

// ---- target-mode level kernels
// Folded constants of the damped Jacobi update and of the Laplacian:
//   v   = om1*C + ax*(E+W) + ay*(N+S) + az*(U+D) + ar*r
//   lap = lx*(E+W) + ly*(N+S) + lz*(U+D) + lc*C
// evaluated with fused multiply-adds; 32-bit offsets (the largest padded level
// array, 515^3 points, is far below 2^31).
template <typename T>
struct TgK {
    T ax, ay, az, ar, om1;
    T lx, ly, lz, lc;
};

template <typename T>
static TgK<T> make_tgk(const Level &L, double omega) {
    TgK<T> k;
    k.ax = (T)(omega * 2.0 * L.cx / L.den);
    k.ay = (T)(omega * 2.0 * L.cy / L.den);
    k.az = (T)(omega * 2.0 * L.cz / L.den);
    k.ar = (T)(-omega * L.c7 / L.den);
    k.om1 = (T)(1.0 - omega);
    k.lx = (T)L.lx; k.ly = (T)L.ly; k.lz = (T)L.lz;
    k.lc = (T)(-2.0 * (L.lx + L.ly + L.lz));
    return k;
}

// Face-ghost images of core point (i, j, k) in the target modes (put_scatter
// without the Dirichlet cases: mirror 1 -> -1, E-1 -> E+1; periodic E-1 -> -1,
// 1 -> E+1), inline: no device call in the caller.
template <typename T>
__device__ __forceinline__ void tgt_images(T *P, int sx, int sy, int i, int j, int k, T v, const MgBC &bc) {
    const long o = (long)(i + 1) * sx + (long)(j + 1) * sy + (k + 1);
    const int q[3] = {i, j, k};
    const long st[3] = {sx, sy, 1};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int E = bc.E[d];
        if (q[d] == 1) P[o + (long)((bc.per[d] ? E + 1 : -1) - 1) * st[d]] = v;
        if (q[d] == E - 1) P[o + (long)((bc.per[d] ? -1 : E + 1) - (E - 1)) * st[d]] = v;
    }
}

template <typename T>
__device__ __noinline__ void scatter_slow(T *P, int sx, int sy, int i, int j, int k, T v, const MgBC &bc) {
    View3<T> V; V.p = P; V.sx = sx; V.sy = sy;
    put_scatter(V, i, j, k, v, bc);
}

// Programmatic dependent launch.  The target-mode level kernels run back to
// back, each a few tens of microseconds at 257^3 and less below; launched with
// programmatic stream serialisation (launch_pdl), the next kernel is launched
// once every block of the previous one has exited, ahead of the grid's
// completion, and waits in pdl_wait, before its first global access, until that
// grid has completed and its writes are visible.  Launched the ordinary way,
// pdl_wait returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... P, typename... A>
static cudaError_t launch_pdl(void (*k)(P...), dim3 g, dim3 b, size_t smem, cudaStream_t st, A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = g;
    cfg.blockDim = b;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

// The target-mode kernels march along x: a (32 k) x (8 j) thread tile walks
// kIch consecutive x planes, keeping the x-1 / x / x+1 values of its column in
// registers, so each point costs one new x-neighbour load plus the four
// in-plane neighbours and the right-hand side.
constexpr int kIch = 8;


static void march_dims(const Level &L, dim3 &g, dim3 &b) {
    b = dim3(32, 8, 1);
    g = dim3((L.n[2] + 1 + 31) / 32, (L.n[1] + 1 + 7) / 8, (L.n[0] + 1 + kIch - 1) / kIch);
}

// Column launches of the marching sweep, residual, prolongation and
// fixed-point residual: one thread per (j, k) column of the core, numbered k
// fastest over the whole (j, k) plane, kColBlock threads a block, blockIdx.y
// the segment of kIch planes.  A level's rows are 2^m + 1 points long, so the
// 32 x 8 tiles of march_dims leave one block in 2^(m-5) + 1 with a single
// active lane per warp.  That costs the FP64 kernels pipe time (a warp
// instruction occupies the FP64 pipe whatever its active lanes; they run at
// its rate on this part), so FP64 launches take columns; the FP32 kernels
// wait on memory instead and keep the tiles, whose in-plane j neighbours
// come from L1 (columns measured 9% slower for the FP32 sweep at 257^3).
constexpr int kColBlock = 256;
static void col_dims(const Level &L, dim3 &g, dim3 &b) {
    long cols = (long)(L.n[1] + 1) * (L.n[2] + 1);
    b = dim3(kColBlock, 1, 1);
    g = dim3((unsigned)((cols + kColBlock - 1) / kColBlock), (L.n[0] + 1 + kIch - 1) / kIch, 1);
}
template <typename T>
static void level_dims(const Level &L, dim3 &g, dim3 &b) {
    if (sizeof(T) == 8) col_dims(L, g, b);
    else march_dims(L, g, b);
}
// The (j, k) column and plane segment of this thread under the launch shape
// of level_dims (COL: columns); false outside the core.
template <bool COL>
__device__ __forceinline__ bool col_of(const MgBC &bc, int &j, int &k, int &seg) {
    if (COL) {
        const int W = bc.E[2] + 1;
        const int t = blockIdx.x * kColBlock + threadIdx.x;
        j = t / W;
        k = t - j * W;
        seg = blockIdx.y;
        return j <= bc.E[1];
    }
    k = blockIdx.x * 32 + threadIdx.x;
    j = blockIdx.y * 8 + threadIdx.y;
    seg = blockIdx.z;
    return j <= bc.E[1] && k <= bc.E[2];
}

// Index of the value a target-mode pad position -1 or E+1 holds: its mirror /
// periodic image in the core (mirror 1 -> -1, E-1 -> E+1; periodic E-1 -> -1,
// 1 -> E+1, the face-ghost images put_scatter writes).
__device__ __forceinline__ int pad_img(int q, int E, int per) {
    if (q < 0) return per ? E - 1 : 1;
    if (q > E) return per ? 1 : E - 1;
    return q;
}

// Neighbour offsets of a (j, k) column of a target-mode level: +-sy and +-1,
// or at a face the offsets of the core images.  The target-mode level kernels
// read the images directly and never the ghost layer, so no kernel has to
// keep face ghosts current between sweeps.
struct NbrJK {
    long yp, ym;   // j + 1, j - 1
    int zp, zm;    // k + 1, k - 1
};
__device__ __forceinline__ NbrJK nbr_jk(int j, int k, int sy, const MgBC &bc) {
    NbrJK n;
    n.yp = (long)(pad_img(j + 1, bc.E[1], bc.per[1]) - j) * sy;
    n.ym = (long)(pad_img(j - 1, bc.E[1], bc.per[1]) - j) * sy;
    n.zp = pad_img(k + 1, bc.E[2], bc.per[2]) - k;
    n.zm = pad_img(k - 1, bc.E[2], bc.per[2]) - k;
    return n;
}
// Offset from plane i to plane i + d (d = +-1), through the image at a face.
__device__ __forceinline__ long nbr_x(int i, int d, int sx, const MgBC &bc) {
    return (long)(pad_img(i + d, bc.E[0], bc.per[0]) - i) * sx;
}

// FP32: __launch_bounds__(256, 6) caps the registers at 40 (six blocks a SM):
// with them the sweep keeps more of a segment's loads in flight than with the
// 32 the compiler picks unbounded (46.5 us against 49.0 a level-0 sweep at
// 257^3; 4 and 5 blocks measured 48.7 and 47.4).  FP64 sweeps wait on the
// FP64 pipe instead; five blocks leave them the registers they took unbounded.
template <typename T, bool ZERO>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 6 : 5) k_tgt_sweep(T *__restrict__ out, const T *__restrict__ in, const T *__restrict__ r,
                                                   int sx, int sy, MgBC bc, TgK<T> c) {
    pdl_wait();
    int j, k, seg;
    if (!col_of<sizeof(T) == 8>(bc, j, k, seg)) return;
    const int i0 = seg * kIch;
    int n = min(kIch, bc.E[0] - i0 + 1);
    const NbrJK nb = nbr_jk(j, k, sy, bc);
    const long o0 = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
    T cm = (T)0, cc = (T)0;
    if (!ZERO) { cm = in[o0 + nbr_x(i0, -1, sx, bc)]; cc = in[o0]; }
    // a full column segment (its planes i0 + 1 .. i0 + kIch are core planes):
    // every load of the segment issued before the first store (the loads are
    // independent of the stores, and issuing them together keeps enough bytes
    // in flight for HBM), then the updates
    if (n == kIch && i0 + kIch <= bc.E[0]) {
        T nc[kIch + 1], ns[kIch], ud[kIch], rr[kIch];
#pragma unroll
        for (int q = 0; q < kIch; ++q) {
            long o = o0 + (long)q * sx;
            nc[q + 1] = ZERO ? (T)0 : in[o + sx];
            ns[q] = ZERO ? (T)0 : in[o + nb.yp] + in[o + nb.ym];
            ud[q] = ZERO ? (T)0 : in[o + nb.zp] + in[o + nb.zm];
            rr[q] = r[o];
        }
        nc[0] = cc;
#pragma unroll
        for (int q = 0; q < kIch; ++q) {
            T v;
            if (ZERO) v = c.ar * rr[q];
            else v = fma(c.ax, cm + nc[q + 1], fma(c.ay, ns[q], fma(c.az, ud[q], fma(c.ar, rr[q], c.om1 * nc[q]))));
            cm = nc[q];
            out[o0 + (long)q * sx] = v;
        }
        return;
    }
    for (int q = 0; q < n; ++q) {
        long o = o0 + (long)q * sx;
        T v;
        if (ZERO) {
            v = c.ar * r[o];
        } else {
            T cp = in[o + nbr_x(i0 + q, 1, sx, bc)];
            T ns = in[o + nb.yp] + in[o + nb.ym], ud = in[o + nb.zp] + in[o + nb.zm];
            v = fma(c.ax, cm + cp, fma(c.ay, ns, fma(c.az, ud, fma(c.ar, r[o], c.om1 * cc))));
            cm = cc;
            cc = cp;
        }
        out[o] = v;
    }
}

// The zero start and the sweep after it in one launch (FP32 levels).  The
// first sweep from 0 is pointwise, s1 = ar1 r (k_tgt_sweep<T, true>), so the
// second reads s1 at its stencil points as ar1 r there: the same FP32 products
// the first launch would have stored, in the same order, so the result is the
// two launches' bits, for 8 bytes a point (r in, iterate out) instead of 20.
template <typename T>
__global__ void __launch_bounds__(256, 6) k_tgt_sweep2z(T *__restrict__ out, const T *__restrict__ r, int sx, int sy, MgBC bc,
                                                       TgK<T> c1, TgK<T> c2) {
    pdl_wait();
    int j, k, seg;
    if (!col_of<sizeof(T) == 8>(bc, j, k, seg)) return;
    const int i0 = seg * kIch;
    const int n = min(kIch, bc.E[0] - i0 + 1);
    const NbrJK nb = nbr_jk(j, k, sy, bc);
    const long o0 = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
    const T a1 = c1.ar;
    T cm = a1 * r[o0 + nbr_x(i0, -1, sx, bc)];
    if (n == kIch && i0 + kIch <= bc.E[0]) {   // a full column segment: every load before the first store
        T nc[kIch + 1], ns[kIch], ud[kIch], rr[kIch];
#pragma unroll
        for (int q = 0; q < kIch; ++q) {
            long o = o0 + (long)q * sx;
            nc[q + 1] = a1 * r[o + sx];
            ns[q] = a1 * r[o + nb.yp] + a1 * r[o + nb.ym];
            ud[q] = a1 * r[o + nb.zp] + a1 * r[o + nb.zm];
            rr[q] = r[o];
        }
        nc[0] = a1 * rr[0];
#pragma unroll
        for (int q = 0; q < kIch; ++q) {
            T v = fma(c2.ax, cm + nc[q + 1], fma(c2.ay, ns[q], fma(c2.az, ud[q], fma(c2.ar, rr[q], c2.om1 * nc[q]))));
            cm = nc[q];
            out[o0 + (long)q * sx] = v;
        }
        return;
    }
    T cc = a1 * r[o0];
    for (int q = 0; q < n; ++q) {
        long o = o0 + (long)q * sx;
        T cp = a1 * r[o + nbr_x(i0 + q, 1, sx, bc)];
        T ns = a1 * r[o + nb.yp] + a1 * r[o + nb.ym], ud = a1 * r[o + nb.zp] + a1 * r[o + nb.zm];
        T v = fma(c2.ax, cm + cp, fma(c2.ay, ns, fma(c2.az, ud, fma(c2.ar, r[o], c2.om1 * cc))));
        cm = cc;
        cc = cp;
        out[o] = v;
    }
}

// Target-mode prolongation + add (vertex-centred trilinear) on the core (the
// target-mode kernels read face neighbours at their images, so no ghost layer
// is written).  A thread owns a fine (j, k)
// column and marches fine planes in pairs: the coarse plane m interpolated to
// (j, k) serves fine plane 2m and, averaged with plane m+1, fine plane 2m+1.
template <typename T>
__global__ void __launch_bounds__(256) k_tgt_prolong_add(T *__restrict__ pf, const T *__restrict__ pc, int sxf, int syf, int sxc, int syc,
                                                         MgBC bc) {
    pdl_wait();
    int j, k, seg;
    if (!col_of<sizeof(T) == 8>(bc, j, k, seg)) return;
    const int i0 = seg * kIch;   // kIch is even
    int iend = min(i0 + kIch - 1, bc.E[0]);
    int k2 = k >> 1, j2 = j >> 1;
    bool ko = k & 1, jo = j & 1;
    auto A = [&](int m) -> T {   // coarse plane m at (j, k)
        const T *q = pc + (long)(m + 1) * sxc + (long)(j2 + 1) * syc + (k2 + 1);
        T v0 = ko ? (T)0.5 * (q[0] + q[1]) : q[0];
        if (!jo) return v0;
        T v1 = ko ? (T)0.5 * (q[syc] + q[syc + 1]) : q[syc];
        return (T)0.5 * (v0 + v1);
    };
    long o = (long)(i0 + 1) * sxf + (long)(j + 1) * syf + (k + 1);
    if (iend - i0 + 1 == kIch) {
        // a full segment: every load issued before the first store (the coarse
        // plane i0 / 2 + kIch / 2 is at most the coarse core's last plane)
        T a[kIch / 2 + 1], v[kIch];
#pragma unroll
        for (int q = 0; q <= kIch / 2; ++q) a[q] = A((i0 >> 1) + q);
#pragma unroll
        for (int q = 0; q < kIch; ++q) v[q] = pf[o + q * (long)sxf];
#pragma unroll
        for (int q = 0; q < kIch; ++q) pf[o + q * (long)sxf] = v[q] + ((q & 1) ? (T)0.5 * (a[q >> 1] + a[(q >> 1) + 1]) : a[q >> 1]);
        return;
    }
    T am = A(i0 >> 1);
    for (int i = i0; i <= iend; i += 2, o += 2 * (long)sxf) {
        pf[o] += am;
        if (i + 1 <= iend) {
            T ap = A((i >> 1) + 1);
            pf[o + sxf] += (T)0.5 * (am + ap);
            am = ap;
        }
    }
}

// r_out = b - Lap(p) over the core; optional max |r| (FP64 accumulation).
template <typename T, typename OT, bool MAXRED>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 6 : 5) k_tgt_residual(OT *__restrict__ out, const T *__restrict__ p, const T *__restrict__ b,
                                                      int sx, int sy, MgBC bc, TgK<T> c, double *maxres) {
    pdl_wait();
    int j, k, seg;
    const bool on = col_of<sizeof(T) == 8>(bc, j, k, seg);
    const int i0 = seg * kIch;
    unsigned long long m = 0ull;
    if (!MAXRED && on && i0 + kIch <= bc.E[0]) {
        // a full column segment (as in k_tgt_sweep): every load before the first store
        const NbrJK nb = nbr_jk(j, k, sy, bc);
        const long o0 = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
        T nc[kIch + 1], ns[kIch], ud[kIch], rr[kIch];
        T cm = p[o0 + nbr_x(i0, -1, sx, bc)];
        nc[0] = p[o0];
#pragma unroll
        for (int q = 0; q < kIch; ++q) {
            long o = o0 + (long)q * sx;
            nc[q + 1] = p[o + sx];
            ns[q] = p[o + nb.yp] + p[o + nb.ym];
            ud[q] = p[o + nb.zp] + p[o + nb.zm];
            rr[q] = b[o];
        }
#pragma unroll
        for (int q = 0; q < kIch; ++q) {
            T lap = fma(c.lx, cm + nc[q + 1], fma(c.ly, ns[q], fma(c.lz, ud[q], c.lc * nc[q])));
            out[o0 + (long)q * sx] = (OT)(rr[q] - lap);
            cm = nc[q];
        }
        return;
    }
    if (on) {
        int iend = min(i0 + kIch - 1, bc.E[0]);
        const NbrJK nb = nbr_jk(j, k, sy, bc);
        long o = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
        T cm = p[o + nbr_x(i0, -1, sx, bc)], cc = p[o];
#pragma unroll 4
        for (int i = i0; i <= iend; ++i, o += sx) {
            T cp = p[o + (i < bc.E[0] ? (long)sx : nbr_x(i, 1, sx, bc))];
            T ns = p[o + nb.yp] + p[o + nb.ym], ud = p[o + nb.zp] + p[o + nb.zm];
            T lap = fma(c.lx, cm + cp, fma(c.ly, ns, fma(c.lz, ud, c.lc * cc)));
            T res = b[o] - lap;
            if (out) out[o] = (OT)res;
            if (MAXRED) {
                unsigned long long a = sizeof(T) == 8 ? abs_bits((double)res) : abs_bits(f2d((float)res));
                m = a > m ? a : m;
            }
            cm = cc;
            cc = cp;
        }
    }
    if (MAXRED) block_max_bits_to(m, maxres);
}

// ---- finest-level FP32 stencils staged through shared memory by the TMA
// The target-mode FP32 Jacobi sweep and residual of the finest level (the
// inner V-cycles of the mixed mode spend most of their HBM traffic there)
// stream x planes of the iterate through a ring of shared-memory slots that
// the Tensor Memory Accelerator fills.  A CTA owns kPlaneRows consecutive j
// rows over the whole k extent (the level's last CTA also its one extra row:
// rows are 2^m + 1 points) and a segment of consecutive i planes.  Rows
// j0-1 .. j0+R of one plane are one contiguous span of the padded level
// array, copied as a 2D box of a tensor map that views the array as rows of
// kPlaneVec floats: the padded row pitch, 2^m + 3 floats, is no multiple of
// 16 bytes, which the strides of a 3D tensor map must be, and 256-byte box
// rows keep the copy engine's requests full.  With the whole k extent in the
// slot, the periodic and mirror images along k are in the slot as well; along
// j the mirror images are in the tile's halo rows and a periodic image row is
// one more box (a second tensor map with a one-row box); along i the slot of
// plane -1 or E+1 holds its image plane.  The right-hand side's rows j0 ..
// j0+R-1 come in the same slot (a third map): a plane of it read from global
// memory into registers one plane ahead waited a full memory latency every
// plane (measured 0.079 ms a 257^3 sweep, against 0.046 for the column kernel).
// Every thread computes; thread 0 also issues the copies and waits on the
// slot's mbarrier.  Plane q goes to slot q % kPlaneRing; after plane i is done
// (one CTA barrier a plane), the slot of plane i - 1 is free and thread 0
// refills it with plane i - 1 + kPlaneRing, so each copy has two planes'
// compute time to land.  The arithmetic is k_tgt_sweep's / k_tgt_residual's, operand for
// operand, so the results are the same bits.
constexpr int kPlaneRows = 8;
constexpr int kPlaneRing = 4;
constexpr int kPlaneVec = 64;        // floats a tensor-map row (256 bytes)
constexpr int kPlaneThreads = 512;

struct PlaneArgs {
    float *out;
    int sx, sy;          // strides of the padded level array, floats
    MgBC bc;
    TgK<float> c;
    int mainRows, sideRows, rRows;   // box heights (rows of kPlaneVec floats) of the three maps
    int sideOff, rOff;   // floats from a slot's start to the side box and the right-hand side's box
    int slotFloats;      // floats a slot
    int planesPerSeg;
    int *err;            // set when an mbarrier wait gives up (1) or the layout is misaligned (2)
};

template <int MODE, int MAXQ>
__global__ void __launch_bounds__(kPlaneThreads, MAXQ <= 5 ? 2 : 1)
    k_tgt_plane_tma(const __grid_constant__ CUtensorMap map, const __grid_constant__ CUtensorMap sideMap,
                    const __grid_constant__ CUtensorMap rMap, const PlaneArgs a) {
    extern __shared__ __align__(128) float plane_sm[];
    __shared__ uint64_t full[kPlaneRing];
    const int tid = threadIdx.x;
    const int E0 = a.bc.E[0], E1 = a.bc.E[1], E2 = a.bc.E[2];
    const int W = E2 + 1, sx = a.sx, sy = a.sy;
    const int nTiles = (E1 + 1) / kPlaneRows;
    const int j0 = blockIdx.x * kPlaneRows;
    const int R = (int)blockIdx.x == nTiles - 1 ? E1 + 1 - j0 : kPlaneRows;
    const int i0 = blockIdx.y * a.planesPerSeg;
    const int i1 = min(i0 + a.planesPerSeg, E0 + 1);
    if (i0 >= i1) return;
    const int nplanes = i1 - i0 + 2;   // planes i0-1 .. i1
    const bool per1 = a.bc.per[1] != 0, per2 = a.bc.per[2] != 0;
    const bool side = per1 && (j0 == 0 || j0 + R - 1 == E1);
    const int sideRow = j0 == 0 ? E1 - 1 : 1;   // periodic image of row -1 / E1 + 1
    const int sideOff = a.sideOff, rOff = a.rOff;
    // slots start at the first 128-byte boundary of the dynamic shared memory
    // (the launch reserves 128 bytes more than the ring)
    float *sm = plane_sm + (((128u - (su32(plane_sm) & 127u)) & 127u) >> 2);
    auto plane_img = [&](int q) { return pad_img(i0 - 1 + q, E0, a.bc.per[0]); };
    // each span is copied from the kPlaneVec-float boundary at or below its
    // start: its data sits at this offset in its box
    auto base = [&](int q) { return (int)((unsigned long)((long)(plane_img(q) + 1) * sx + (long)j0 * sy) & (kPlaneVec - 1)); };
    auto side_base = [&](int q) { return (int)((unsigned long)((long)(plane_img(q) + 1) * sx + (long)(sideRow + 1) * sy) & (kPlaneVec - 1)); };
    auto r_base = [&](int q) { return (int)((unsigned long)((long)(plane_img(q) + 1) * sx + (long)(j0 + 1) * sy) & (kPlaneVec - 1)); };
    const uint32_t tx = (uint32_t)((a.mainRows + a.rRows + (side ? a.sideRows : 0)) * kPlaneVec * 4);
    int issued = 0;   // thread 0: planes whose copies are issued
    auto issue = [&](int q) {
        const int slot = q % kPlaneRing, ii = plane_img(q);
        uint64_t *m = &full[slot];
        const uint32_t dst = su32(sm + (size_t)slot * a.slotFloats);
        mbar_arrive_expect_tx(m, tx);
        tma_load_2d(dst, &map, 0, (int)(((long)(ii + 1) * sx + (long)j0 * sy) / kPlaneVec), m);   // array row j0: row j0 - 1
        if (side) tma_load_2d(dst + sideOff * 4, &sideMap, 0, (int)(((long)(ii + 1) * sx + (long)(sideRow + 1) * sy) / kPlaneVec), m);
        tma_load_2d(dst + rOff * 4, &rMap, 0, (int)(((long)(ii + 1) * sx + (long)(j0 + 1) * sy) / kPlaneVec), m);
        issued = q + 1;
    };
    bool ok = true;
    if (tid == 0) {
        // every box lands at a 128-byte aligned address (the layout's
        // invariant, checked so that a bad layout reports instead of issuing
        // a misaligned copy)
        if (((su32(sm) | (uint32_t)(a.slotFloats * 4) | (uint32_t)(sideOff * 4) | (uint32_t)(rOff * 4)) & 127u) != 0u) {
            atomicExch(a.err, 2);
            ok = false;
        }
        for (int q = 0; q < kPlaneRing; ++q) mbar_init(&full[q], 1);
        fence_mbar_init();
        if (ok) {
            for (int q = 0; q < kPlaneRing && q < nplanes; ++q) issue(q);
            for (int q = 0; q < 3 && ok; ++q) ok = mbar_wait(&full[q], 0, a.err);   // planes i0-1, i0, i0+1
        }
    }
    if (__syncthreads_or(!ok)) {
        if (tid == 0)   // leave no copy in flight (bounded)
            for (int w = 0; w < issued; ++w) mbar_wait(&full[w % kPlaneRing], (w / kPlaneRing) & 1, nullptr);
        return;
    }
    // this thread's points of a plane, p = tid + 512 q over the tile's R x W points
    const int npts = R * W;
    int P[MAXQ];   // the point's index in a slot after the plane's base offset (row 0 of a slot is row j0 - 1)
    unsigned edge = 0u, live = 0u;
#pragma unroll
    for (int q = 0; q < MAXQ; ++q) {
        const int p = tid + q * kPlaneThreads;
        const int row = p / W, col = p - row * W;
        P[q] = (row + 1) * sy + col + 1;
        if (p < npts) live |= 1u << q;
        if (p < npts && (col == 0 || col == E2 || j0 + row == 0 || j0 + row == E1)) edge |= 1u << q;
    }
    const int gj = j0 * sy;
    const TgK<float> &c = a.c;
    // slot pointers (after each plane's base offset) of planes qc - 1, qc, qc + 1, rolled along
    const float *sp = sm + base(0), *sc = sm + (size_t)a.slotFloats + base(1), *sn = sm + (size_t)2 * a.slotFloats + base(2);
    int slotC = 1;
    for (int i = i0; i < i1; ++i) {
        const int qc = i - i0 + 1;   // plane i is plane qc of the segment
        const float *scs = sm + (size_t)slotC * a.slotFloats;
        const float *ss = side ? scs + sideOff + side_base(qc) : scs;
        const float *sr = scs + rOff + r_base(qc) - sy;   // P[q] counts rows from j0 - 1
        float *out = a.out + (long)(i + 1) * sx + gj;
#pragma unroll
        for (int q = 0; q < MAXQ; ++q) {
            if (!((live >> q) & 1u)) continue;
            const int x = P[q];
            const float C = sc[x], Wv = sp[x], Ev = sn[x], rv = sr[x];
            float N, S, U, D;
            if (!((edge >> q) & 1u)) {
                N = sc[x + sy]; S = sc[x - sy]; U = sc[x + 1]; D = sc[x - 1];
            } else {
                const int p = tid + q * kPlaneThreads;
                const int row = p / W, col = p - row * W, j = j0 + row;
                N = j == E1 ? (per1 ? ss[col + 1] : sc[x - sy]) : sc[x + sy];
                S = j == 0 ? (per1 ? ss[col + 1] : sc[x + sy]) : sc[x - sy];
                U = col == E2 ? (per2 ? sc[x + 1 - E2] : sc[x - 1]) : sc[x + 1];
                D = col == 0 ? (per2 ? sc[x + E2 - 1] : sc[x + 1]) : sc[x - 1];
            }
            float v;
            if (MODE == 0) {
                v = fmaf(c.ax, Wv + Ev, fmaf(c.ay, N + S, fmaf(c.az, U + D, fmaf(c.ar, rv, c.om1 * C))));
            } else {
                const float lap = fmaf(c.lx, Wv + Ev, fmaf(c.ly, N + S, fmaf(c.lz, U + D, c.lc * C)));
                v = rv - lap;
            }
            out[x] = v;
        }
        // one barrier a plane: every thread is done with plane qc - 1 (its slot
        // takes plane qc - 1 + kPlaneRing), and thread 0 has seen plane qc + 2,
        // which the next plane reads, land
        if (tid == 0 && qc + 2 < nplanes) ok = mbar_wait(&full[(qc + 2) % kPlaneRing], ((qc + 2) / kPlaneRing) & 1, a.err);
        if (__syncthreads_or(!ok)) break;
        if (tid == 0 && qc - 1 + kPlaneRing < nplanes) {
            fence_async_smem();
            issue(qc - 1 + kPlaneRing);
        }
        slotC = slotC + 1 == kPlaneRing ? 0 : slotC + 1;
        const int slotN = slotC + 1 == kPlaneRing ? 0 : slotC + 1;
        sp = sc;
        sc = sn;
        sn = sm + (size_t)slotN * a.slotFloats + (qc + 2 < nplanes ? base(qc + 2) : 0);
    }
    // leave no copy in flight: every issued plane's slot complete (bounded) before the CTA ends
    if (tid == 0)
        for (int w = max(0, issued - kPlaneRing); w < issued; ++w) mbar_wait(&full[w % kPlaneRing], (w / kPlaneRing) & 1, nullptr);
}

// Full-weighting restriction of a target-mode residual (k_mg_restrict's
// weights (1/64) [1 2 1]^3, summed separably): one thread per coarse (J, K)
// column (column launch, k fastest over the coarse plane) marching rr_ch
// coarse planes along I; each fine plane's in-plane
// [1 2 1] x [1 2 1] sum is formed once and the odd fine plane between two
// coarse planes serves both.  Fine positions outside the core are read at
// their mirror / periodic images (the pads k_mg_restrict resolves).
// Coarse planes per thread: FP32 restrictions wait on memory and keep
// longer chains (each odd fine plane serves two coarse planes); FP64 ones
// are bound by the FP64 pipe and want more threads (measured at 257^3).
template <typename T>
constexpr int rr_ch() { return sizeof(T) == 8 ? 4 : 8; }
// __launch_bounds__(256, 4): up to 64 registers, so a thread's loads of the
// next fine planes are in flight together (FP32 257^3: 24.0 us against 27.0
// with the compiler's unbounded choice of 32 registers).


template <typename T>
__global__ void __launch_bounds__(256, 4) k_tgt_restrict(T *__restrict__ rc, const T *__restrict__ r, int sx, int sy, int csx, int csy,
                                                       MgBC bcf) {
    pdl_wait();
    const int E0 = bcf.E[0], E1 = bcf.E[1], E2 = bcf.E[2];
    const int W = E2 / 2 + 1, t = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = t / W, K = t - J * W, I0 = blockIdx.y * rr_ch<T>();
    if (J > E1 / 2) return;
    long oj[3];
    int ok[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        oj[a] = (long)(pad_img(2 * J - 1 + a, E1, bcf.per[1]) + 1) * sy;
        ok[a] = pad_img(2 * K - 1 + a, E2, bcf.per[2]) + 1;
    }
    auto plane = [&](int i) -> T {
        const T *q = r + (long)(pad_img(i, E0, bcf.per[0]) + 1) * sx;
        T row[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const T *qa = q + oj[a];
            row[a] = qa[ok[0]] + (T)2 * qa[ok[1]] + qa[ok[2]];
        }
        return row[0] + (T)2 * row[1] + row[2];
    };
    const int Iend = min(I0 + rr_ch<T>() - 1, E0 / 2);
    T lo = plane(2 * I0 - 1);
#pragma unroll 2
    for (int I = I0; I <= Iend; ++I) {
        T mid = plane(2 * I), hi = plane(2 * I + 1);
        rc[(long)(I + 1) * csx + (long)(J + 1) * csy + (K + 1)] = (lo + (T)2 * mid + hi) * (T)0.015625;
        lo = hi;
    }
}

// p64 += e32 over the core (FP64 correction accumulation) with face ghosts.
__global__ void __launch_bounds__(256) k_tgt_update(double *__restrict__ p, const float *__restrict__ e, int sx, int sy, MgBC bc) {
    int k = blockIdx.x * 32 + threadIdx.x;
    int j = blockIdx.y * 8 + threadIdx.y;
    int i0 = blockIdx.z * kIch;
    if (j > bc.E[1] || k > bc.E[2]) return;
    int iend = min(i0 + kIch - 1, bc.E[0]);
    int o = (i0 + 1) * sx + (j + 1) * sy + (k + 1);
    bool edge_jk = j <= 1 || k <= 1 || j >= bc.E[1] - 1 || k >= bc.E[2] - 1;
#pragma unroll 4
    for (int i = i0; i <= iend; ++i, o += sx) {
        double v = p[o] + (double)e[o];
        p[o] = v;
        if (edge_jk || i <= 1 || i >= bc.E[0] - 1) scatter_slow(p, sx, sy, i, j, k, v, bc);
    }
}

// ---- exact fixed-point refinement (SARAS_MG_MIXED, isotropic level 0)
// With lx = ly = lz = l the level-0 residual is r = b - l (sum of the six
// neighbours - 6 centre).  Holding the iterate as integers P = round(p 2^s) and
// the right-hand side as B = round(b 2^s / l) makes it
//     r = l 2^-s (B - (sum of the six neighbours of P - 6 P)),
// evaluated exactly in 64-bit integer arithmetic: no rounding at all, where an
// FP64 residual loses the digits the stencil cancels (about log10 of
// (N / pi)^2 of them for smooth fields).  s is chosen per solve so that
// |P|, |B| <= 2^55; sums of seven terms stay below 2^59.  GB300 runs these
// integer operations at the FP32 rate, 64 times its FP64 rate, so the
// residual is bound by HBM.
//
// k_fx_refine: the residual of P; r32 receives r in FP32 (the next V-cycle's
// right-hand side), maxr the block maxima of |B - ...| in integer units.
// Neighbours at the faces are read at their core images (nbr_jk, nbr_x).
// P rounded to the 53 significant bits of an FP64 value (to nearest, ties to
// even): the fixed-point value of the FP64 number P 2^-s that k_fx_output
// writes (the scaling by 2^-s is exact), from integer operations only.
__device__ __forceinline__ long long round53(long long p) {
    unsigned long long a = p < 0 ? 0ull - (unsigned long long)p : (unsigned long long)p;
    if (a < (1ull << 53)) return p;
    int sh = 11 - __clzll((long long)a);   // bits below the 53 kept: 64 - clz - 53
    unsigned long long low = a & ((1ull << sh) - 1), half = 1ull << (sh - 1), q = a >> sh;
    if (low > half || (low == half && (q & 1ull))) q += 1;
    a = q << sh;
    return p < 0 ? -(long long)a : (long long)a;
}

__global__ void __launch_bounds__(256) k_fx_refine(const long long *__restrict__ pin, const long long *__restrict__ bfx,
                                                   float *__restrict__ r32, int sx, int sy, MgBC bc, float rscale,
                                                   unsigned long long *maxr) {
    int j, k, seg;
    const bool on = col_of<true>(bc, j, k, seg);
    const int i0 = seg * kIch;
    unsigned long long m = 0;
    if (on) {
        int iend = min(i0 + kIch - 1, bc.E[0]);
        const NbrJK nb = nbr_jk(j, k, sy, bc);
        long o = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
        long long cm = pin[o + nbr_x(i0, -1, sx, bc)], cc = pin[o];
        for (int i = i0; i <= iend; ++i, o += sx) {
            long long cp = pin[o + (i < bc.E[0] ? (long)sx : nbr_x(i, 1, sx, bc))];
            long long nsum = (cm + cp) + (pin[o + nb.yp] + pin[o + nb.ym]) + (pin[o + nb.zp] + pin[o + nb.zm]);
            long long r = bfx[o] - (nsum - 6 * cc);
            if (r32) r32[o] = fx2f(r) * rscale;
            unsigned long long a = (unsigned long long)(r < 0 ? -r : r);
            m = a > m ? a : m;
            cm = cc;
            cc = cp;
        }
    }
    block_max_bits_to(m, reinterpret_cast<double *>(maxr));
}

// The iterate advanced by the FP32 correction e of the inner V-cycles,
// P_out = round53(P_in + round(e 2^s)) (so that every iterate is a value FP64
// holds exactly: P_out 2^-s is the solve's FP64 output, written to dst at the
// core points when dst is given), and the residual of P_out (as k_fx_refine),
// which is then the exact residual of that output; with
// the in-plane neighbours shared through shared memory: each advanced value is
// formed once per block (the tile's halo adds a third), instead of once per
// stencil use.  Block 32 (k) x 8 (j) marching kIch planes along i; the plane
// tiles rotate through three buffers (one barrier a plane), tile positions and
// planes outside the core are read at their images, and the column's own
// i - 1 / i + 1 values stay in registers.  flag: a value outside the
// fixed-point range.
__global__ void __launch_bounds__(256, 8) k_fx_update(long long *__restrict__ pout, const long long *__restrict__ pin,
                                                   const float *__restrict__ e, const long long *__restrict__ bfx,
                                                   float *__restrict__ r32, int sx, int sy, MgBC bc, int s, float rscale,
                                                   unsigned long long *maxr, int *flag, double *__restrict__ dst, double inv2s) {
    __shared__ long long tile[3][10][34];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int k0 = blockIdx.x * 32, j0 = blockIdx.y * 8, i0 = blockIdx.z * kIch;
    const int k = k0 + tx, j = j0 + ty;
    const int iend = min(i0 + kIch - 1, bc.E[0]);
    bool bad = false;
    auto val = [&](long q) -> long long { return round53(pin[q] + f2fx(e[q], s, bad)); };
    // the two tile positions this thread loads: (j0 - 1 .. j0 + 8, k0 - 1 .. k0 + 32)
    long lo[2];
    bool lv[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        int t = tid + 256 * q;
        int jj = t / 34, kk = t - jj * 34;
        int jg = j0 + jj - 1, kg = k0 + kk - 1;
        lv[q] = t < 340 && jg <= bc.E[1] + 1 && kg <= bc.E[2] + 1;
        lo[q] = (long)(pad_img(jg, bc.E[1], bc.per[1]) + 1) * sy + (pad_img(kg, bc.E[2], bc.per[2]) + 1);
    }
    auto load_plane = [&](int i, int buf) {
        long base = (long)(pad_img(i, bc.E[0], bc.per[0]) + 1) * sx;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            int t = tid + 256 * q;
            if (t < 340) (&tile[buf][0][0])[t] = lv[q] ? val(base + lo[q]) : 0;
        }
    };
    unsigned long long m = 0;
    if ((bc.E[2] & 31) == 0 && bc.E[2] >= 32 && blockIdx.x == gridDim.x - 1) {
        // the tiles of rows of 32 m + 1 points leave their last column (k = E2) to
        // a tile of one live lane; here it is dealt densely, a (j, segment) column
        // a thread over the last block column, operands read at their images from
        // global memory (integer sums: the tiles' values)
        const long t = ((long)blockIdx.z * gridDim.y + blockIdx.y) * 256 + tid;
        const int W = bc.E[1] + 1;
        if (t < (long)W * gridDim.z) {
            const int je = (int)(t % W), ie0 = (int)(t / W) * kIch, ke = bc.E[2];
            const int ie1 = min(ie0 + kIch - 1, bc.E[0]);
            const NbrJK nb = nbr_jk(je, ke, sy, bc);
            long oe = (long)(ie0 + 1) * sx + (long)(je + 1) * sy + (ke + 1);
            long long em = val(oe + nbr_x(ie0, -1, sx, bc));
            for (int i = ie0; i <= ie1; ++i, oe += sx) {
                const long long cc = val(oe), cp = val(oe + nbr_x(i, 1, sx, bc));
                const long long nsum = (em + cp) + (val(oe + nb.ym) + val(oe + nb.yp)) + (val(oe + nb.zm) + val(oe + nb.zp));
                const long long r = bfx[oe] - (nsum - 6 * cc);
                r32[oe] = fx2f(r) * rscale;
                const unsigned long long a = (unsigned long long)(r < 0 ? -r : r);
                m = a > m ? a : m;
                pout[oe] = cc;
                if (dst) dst[oe] = __ll2double_rn(cc) * inv2s;
                const unsigned long long ac = (unsigned long long)(cc < 0 ? -cc : cc);
                if (ac > (1ull << 59)) bad = true;
                em = cc;
            }
        }
    } else {
    const bool active = j <= bc.E[1] && k <= bc.E[2];
    long o = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
    long long cm = active ? val(o + nbr_x(i0, -1, sx, bc)) : 0;
    load_plane(i0, 0);
    for (int i = i0; i <= iend; ++i, o += sx) {
        const int b = (i - i0) % 3, bn = (i - i0 + 1) % 3;
        load_plane(i + 1, bn);
        __syncthreads();
        if (active) {
            long long cc = tile[b][ty + 1][tx + 1], cp = tile[bn][ty + 1][tx + 1];
            long long nsum = (cm + cp) + (tile[b][ty][tx + 1] + tile[b][ty + 2][tx + 1]) + (tile[b][ty + 1][tx] + tile[b][ty + 1][tx + 2]);
            long long r = bfx[o] - (nsum - 6 * cc);
            r32[o] = fx2f(r) * rscale;
            unsigned long long a = (unsigned long long)(r < 0 ? -r : r);
            m = a > m ? a : m;
            pout[o] = cc;
            if (dst) dst[o] = __ll2double_rn(cc) * inv2s;
            unsigned long long ac = (unsigned long long)(cc < 0 ? -cc : cc);
            if (ac > (1ull << 59)) bad = true;
            cm = cc;
        }
    }
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        unsigned long long o2 = __shfl_xor_sync(0xffffffffu, m, off);
        m = o2 > m ? o2 : m;
    }
    __shared__ unsigned long long sm[8];
    if (tx == 0) sm[ty] = m;
    __syncthreads();
    if (tid == 0) {
        unsigned long long bm = 0;
        for (int q = 0; q < 8; ++q) bm = sm[q] > bm ? sm[q] : bm;
        atomicMax(maxr, bm);
    }
    if (bad) atomicExch(flag, 1);
}

// The fixed-point iterate straight from the previous Pp: core points with
// their face-ghost images (k_mg_init_p's put_scatter), no FP64 level copy.
__global__ void k_fx_init(long long *__restrict__ dst, View3<const double> src, MgBC bc, int s, int *flag) {
    int i, j, k;
    if (!core_pt(bc.E, i, j, k)) return;
    bool bad = false;
    View3<long long> V;
    V.p = dst; V.sx = src.sx; V.sy = src.sy;
    put_scatter(V, i, j, k, d2fx(src(i, j, k), s, bad), bc);
    if (bad) atomicExch(flag, 1);
}

// The solve's output written straight into Pp: every padded point takes the
// value of the core point the imposeBC composition maps it to (k_mg_output's
// mapping, target modes: periodic or mirror per axis), P 2^-s.  Every
// fixed-point iterate is a value FP64 holds exactly (an FP64 value scaled by
// 2^s, or round53 in k_fx_update), so the conversion is exact and the
// iterate's residual is the exact residual of what the solve returns.  One
// thread per point of a (k, j) row, blockIdx.z the plane.
__global__ void k_fx_output(double *__restrict__ dst, const long long *__restrict__ src, MgBC bc, double inv2s) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x - 1, j = blockIdx.y * blockDim.y + threadIdx.y - 1, i = blockIdx.z - 1;
    const int E1 = bc.E[1], E2 = bc.E[2];
    if (j > E1 + 1 || k > E2 + 1) return;
    const long sy = E2 + 3, sx = (long)(E1 + 3) * sy;
    int q[3] = {i, j, k};
    for (int d = 2; d >= 0; --d) {
        int E = bc.E[d];
        if (q[d] >= 0 && q[d] <= E) continue;
        if (bc.per[d]) q[d] = q[d] < 0 ? E - 1 : 1;
        else q[d] = q[d] < 0 ? 1 : E - 1;
    }
    const long o = (i + 1) * sx + (j + 1) * sy + (k + 1);
    dst[o] = __ll2double_rn(src[(q[0] + 1) * sx + (q[1] + 1) * sy + (q[2] + 1)]) * inv2s;
}

// The ghost positions of the output Pp (k_fx_output's mapping) once the
// core holds P 2^-s: blockIdx.z the face (axis z / 2, low or high side),
// threads over that face's padded positions.  Points on edges and corners
// are written by every face they lie on, with one value.
__global__ void k_fx_output_shell(double *__restrict__ dst, const long long *__restrict__ src, MgBC bc, double inv2s) {
    const int d = blockIdx.z >> 1, side = blockIdx.z & 1;
    const int a = (d + 1) % 3, b = (d + 2) % 3;
    const int na = bc.E[a] + 3, nb = bc.E[b] + 3;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na * nb) return;
    int q[3];
    q[d] = side ? bc.E[d] + 1 : -1;
    q[a] = t / nb - 1;
    q[b] = t - (q[a] + 1) * nb - 1;
    const long sy = bc.E[2] + 3, sx = (long)(bc.E[1] + 3) * sy;
    const long o = (q[0] + 1) * sx + (q[1] + 1) * sy + (q[2] + 1);
    for (int e = 0; e < 3; ++e) {
        int E = bc.E[e];
        if (q[e] >= 0 && q[e] <= E) continue;
        if (bc.per[e]) q[e] = q[e] < 0 ? E - 1 : 1;
        else q[e] = q[e] < 0 ? 1 : E - 1;
    }
    dst[o] = __ll2double_rn(src[(q[0] + 1) * sx + (q[1] + 1) * sy + (q[2] + 1)]) * inv2s;
}

// B = round((rhs - mean) mul) over the core (mul = 2^s / l; the residual reads
// B only there), and, with bout, b = rhs - mean itself (the FP64 right-hand
// side that the restricted histories and the FP64 fallback read).  Column
// launch.
__global__ void __launch_bounds__(256) k_fx_rhs(long long *__restrict__ dst, double *__restrict__ bout, const double *__restrict__ rhs,
                                                int sx, int sy, MgBC bc, double mean, double mul, int *flag) {
    int j, k, seg;
    if (!col_of<true>(bc, j, k, seg)) return;
    const int i0 = seg * kIch, iend = min(i0 + kIch - 1, bc.E[0]);
    long o = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
    bool bad = false;
    for (int i = i0; i <= iend; ++i, o += sx) {
        const double b = rhs[o] - mean;
        if (bout) bout[o] = b;
        dst[o] = d2fx(b * mul, 0, bad);
    }
    if (bad) atomicExch(flag, 1);
}


// ---- target modes (FP64 / mixed)
// Order-preserving key of a double (unsigned comparison of keys = numeric
// comparison of values, NaN above +Inf), and its inverse on the host.
__device__ __forceinline__ unsigned long long order_key(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
static double order_key_value(unsigned long long key) {
    unsigned long long b = (key >> 63) ? (key & 0x7fffffffffffffffull) : ~key;
    double v;
    std::memcpy(&v, &b, sizeof v);
    return v;
}

// The inputs of a target-mode solve in one pass over the core: trapezoidal-
// weight partial sums of rhs (one per block, in block order), max and min of
// rhs (keys: max |rhs - mean| = max(max - mean, mean - min), exactly, as
// rounding is monotone), and with pp, max |pp| (the fixed-point scale).
// Column launch.
__global__ void __launch_bounds__(256) k_tgt_stats(View3<const double> rhs, const double *__restrict__ pp, MgBC bc, double *part,
                                                   double *kmax, double *kmin, double *pmax) {
    __shared__ double sm[8];
    int j, k, seg;
    const bool on = col_of<true>(bc, j, k, seg);
    // weight 2^-(number of axes on which the point is an end point), as one
    // table lookup: the product of three halves costs GB300's FP64 pipe
    const double wt[4] = {1.0, 0.5, 0.25, 0.125};
    double s = 0;
    unsigned long long hi = 0, lo = 0, pm = 0;
    if (on) {
        const int ejk = (j == 0 || j == bc.E[1]) + (k == 0 || k == bc.E[2]);
        const int i0 = seg * kIch, iend = min(i0 + kIch - 1, bc.E[0]);
        long o = (long)(i0 + 1) * rhs.sx + (long)(j + 1) * rhs.sy + (k + 1);
        for (int i = i0; i <= iend; ++i, o += rhs.sx) {
            const double v = rhs.p[o];
            s = fma(wt[ejk + (i == 0 || i == bc.E[0])], v, s);
            const unsigned long long key = order_key(v);
            hi = key > hi ? key : hi;
            lo = ~key > lo ? ~key : lo;
            if (pp) {
                const unsigned long long a = abs_bits(pp[o]);
                pm = a > pm ? a : pm;
            }
        }
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) S += sm[w];
        part[(long)blockIdx.y * gridDim.x + blockIdx.x] = S;
    }
    block_max_bits_to(hi, kmax);
    block_max_bits_to(lo, kmin);
    if (pp) block_max_bits_to(pm, pmax);
}

// b = rhs - mean over the core (the FP64 right-hand side).  Column launch.
__global__ void __launch_bounds__(256) k_tgt_rhs(double *__restrict__ b, const double *__restrict__ rhs, int sx, int sy, MgBC bc,
                                                 double mean) {
    int j, k, seg;
    if (!col_of<true>(bc, j, k, seg)) return;
    const int i0 = seg * kIch, iend = min(i0 + kIch - 1, bc.E[0]);
    long o = (long)(i0 + 1) * sx + (long)(j + 1) * sy + (k + 1);
    for (int i = i0; i <= iend; ++i, o += sx) b[o] = rhs[o] - mean;
}

// ---- the coarse end of a target-mode V-cycle in one CTA
// Levels Lt..depth (at most kTailIntervals intervals per axis at Lt) fit in
// shared memory together; at these sizes their sweeps, residuals and
// transfers are launch-latency bound, and the coarsest Gauss-Seidel loop runs
// on one CTA anyway.  k_mg_tail runs that whole sub-cycle: pre-smoothing from zero and
// restriction down to the coarsest level, the coarsest solve (coarse_gs),
// prolongation and post-smoothing back up to Lt, with the kernels' arithmetic
// (k_tgt_sweep, k_tgt_residual, k_mg_restrict, k_mg_prolong_add), and writes
// the level-Lt iterate with its face-ghost images to global memory.
constexpr int kTailMaxLevels = 8;
// The tail's first level: 9^3 at most.  One CTA runs a 17^3 level's Chebyshev
// sweeps instruction-bound on one SM; graph-replayed kernels on all SMs ran
// the 257^3 steps 0.7% (mixed) and 3% (plain FP64) faster with 17^3 outside
// the tail.
constexpr int kTailIntervals = 8;
constexpr int kTailMaxSweeps = 16;
constexpr int kTailThreads = 1024;

template <typename T>
struct TailArgs {
    int nl;                          // levels in the tail: Lt .. Lt + nl - 1 (the coarsest)
    MgBC bc[kTailMaxLevels];
    TgK<T> tk[kTailMaxLevels];       // sweep constants at weight 1 (scaled per sweep by wpre / wpost)
    T wpre[kTailMaxSweeps], wpost[kTailMaxSweeps];   // sweep weights (smooth_weight)
    TgK<T> tr[kTailMaxLevels];       // residual constants (weight 1)
    MgK kkc;                         // coarsest level (Gauss-Seidel)
    const T *M;                      // coarsest solution operator (nM x nM), or null: Gauss-Seidel
    int nM;
    T tol;
    int maxc, pre, post;
    const T *rin;                    // level-Lt right-hand side (padded)
    T *pout;                         // level-Lt iterate (padded)
    long long *iters;
};

template <typename T>
__device__ __forceinline__ int tail_count(const MgBC &b) { return (b.E[0] + 3) * (b.E[1] + 3) * (b.E[2] + 3); }

// The core points (i, j, k) of an (X1 x Y1 x Z1)-point level, k fastest, that
// thread t visits at t, t + nt, ...: the first point by division, the others
// by adding the stride nt in mixed radix (one carry per digit at most, since
// each digit of the stride is below its radix), so the loop body is free of
// integer divisions.
template <typename F>
__device__ __forceinline__ void tail_for(int X1, int Y1, int Z1, F f) {
    const int nt = blockDim.x, n = X1 * Y1 * Z1, YZ = Y1 * Z1;
    int t = threadIdx.x;
    if (t >= n) return;
    int i = t / YZ, r = t - i * YZ, j = r / Z1, k = r - j * Z1;
    const int di = nt / YZ, rr = nt - di * YZ, dj = rr / Z1, dk = rr - dj * Z1;
    for (; t < n; t += nt) {
        f(i, j, k);
        k += dk;
        if (k >= Z1) { k -= Z1; ++j; }
        j += dj;
        if (j >= Y1) { j -= Y1; ++i; }
        i += di;
    }
}

template <typename T>
__device__ __forceinline__ bool near_face(int i, int j, int k, const MgBC &bc) {
    return i <= 1 || j <= 1 || k <= 1 || i >= bc.E[0] - 1 || j >= bc.E[1] - 1 || k >= bc.E[2] - 1;
}

// The sweep constants at weight w from those at weight 1.
template <typename T>
__device__ __forceinline__ TgK<T> tgk_weight(const TgK<T> &c1, T w) {
    TgK<T> c = c1;
    c.ax = w * c1.ax; c.ay = w * c1.ay; c.az = w * c1.az; c.ar = w * c1.ar;
    c.om1 = (T)1 - w;
    return c;
}

template <typename T, bool ZERO>
__device__ void tail_sweep(T *out, const T *in, const T *r, const MgBC &bc, const TgK<T> &c) {
    const int E1 = bc.E[1], E2 = bc.E[2], sy = E2 + 3, sx = (E1 + 3) * sy;
    tail_for(bc.E[0] + 1, E1 + 1, E2 + 1, [&](int i, int j, int k) {
        int o = (i + 1) * sx + (j + 1) * sy + (k + 1);
        T v;
        if (ZERO) v = c.ar * r[o];
        else v = fma(c.ax, in[o - sx] + in[o + sx], fma(c.ay, in[o + sy] + in[o - sy], fma(c.az, in[o + 1] + in[o - 1], fma(c.ar, r[o], c.om1 * in[o]))));
        out[o] = v;
        if (near_face<T>(i, j, k, bc)) tgt_images(out, sx, sy, i, j, k, v, bc);
    });
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kTailThreads) k_mg_tail(TailArgs<T> a) {
    pdl_wait();
    extern __shared__ unsigned char smraw[];
    T *base = reinterpret_cast<T *>(smraw);
    T *P[kTailMaxLevels], *Q[kTailMaxLevels], *R[kTailMaxLevels];
    {
        T *q = base;
        for (int l = 0; l < a.nl; ++l) {
            int n = tail_count<T>(a.bc[l]);
            P[l] = q; Q[l] = q + n; R[l] = q + 2 * n;
            q += 3 * n;
        }
    }
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int t = tid; t < tail_count<T>(a.bc[0]); t += nt) R[0][t] = a.rin[t];
    __syncthreads();
    for (int l = 0; l + 1 < a.nl; ++l) {
        const MgBC &bc = a.bc[l];
        int E1 = bc.E[1], E2 = bc.E[2], sy = E2 + 3, sx = (E1 + 3) * sy;
        // pre-smoothing from zero (the first sweep ignores its input)
        for (int n = 0; n < a.pre; ++n) {
            const TgK<T> cw = tgk_weight(a.tk[l], a.wpre[n]);
            if (n == 0) tail_sweep<T, true>(Q[l], P[l], R[l], bc, cw);
            else tail_sweep<T, false>(Q[l], P[l], R[l], bc, cw);
            T *x = P[l]; P[l] = Q[l]; Q[l] = x;
        }
        // residual into Q (core), then full-weighting restriction (k_tgt_restrict's
        // separable form; fine positions outside the core at their images)
        const TgK<T> &c = a.tr[l];
        {
            const T *p = P[l], *rr = R[l];
            T *qq = Q[l];
            tail_for(bc.E[0] + 1, E1 + 1, E2 + 1, [&](int i, int j, int k) {
                int o = (i + 1) * sx + (j + 1) * sy + (k + 1);
                T lap = fma(c.lx, p[o - sx] + p[o + sx], fma(c.ly, p[o + sy] + p[o - sy], fma(c.lz, p[o + 1] + p[o - 1], c.lc * p[o])));
                qq[o] = rr[o] - lap;
            });
        }
        __syncthreads();
        const MgBC &bcc = a.bc[l + 1];
        int C1 = bcc.E[1], C2 = bcc.E[2], csy = C2 + 3, csx = (C1 + 3) * csy;
        {
            const T *qf = Q[l];
            T *rc = R[l + 1];
            tail_for(bcc.E[0] + 1, C1 + 1, C2 + 1, [&](int I, int J, int K) {
                int oj[3], ok[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    oj[q] = (pad_img(2 * J - 1 + q, E1, bc.per[1]) + 1) * sy;
                    ok[q] = pad_img(2 * K - 1 + q, E2, bc.per[2]) + 1;
                }
                T acc = (T)0;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const T *pl = qf + (pad_img(2 * I - 1 + q, bc.E[0], bc.per[0]) + 1) * sx;
                    T row[3];
#pragma unroll
                    for (int w = 0; w < 3; ++w) {
                        const T *pr = pl + oj[w];
                        row[w] = pr[ok[0]] + (T)2 * pr[ok[1]] + pr[ok[2]];
                    }
                    T sp = row[0] + (T)2 * row[1] + row[2];
                    acc += q == 1 ? (T)2 * sp : sp;
                }
                rc[(I + 1) * csx + (J + 1) * csy + (K + 1)] = acc * (T)0.015625;
            });
        }
        __syncthreads();
    }
    // coarsest level: e = M r with the precomputed solution operator (one warp
    // per row, the core right-hand side gathered into a compact vector first),
    // else Gauss-Seidel to tol
    {
        int L = a.nl - 1;
        const MgBC &bc = a.bc[L];
        for (int t = tid; t < tail_count<T>(bc); t += nt) P[L][t] = (T)0;
        if (a.M) {
            int Y = bc.E[1], Z = bc.E[2], sy = Z + 3, sx = (Y + 3) * sy;
            T *rv = Q[L];
            const T *rl = R[L];
            tail_for(bc.E[0] + 1, Y + 1, Z + 1, [&](int i, int j, int k) {
                rv[(i * (Y + 1) + j) * (Z + 1) + k] = rl[(i + 1) * sx + (j + 1) * sy + (k + 1)];
            });
            __syncthreads();
            int lane = tid & 31;
            for (int row = tid >> 5; row < a.nM; row += nt >> 5) {
                const T *m = a.M + (long)row * a.nM;
                T s = (T)0;
                for (int q = lane; q < a.nM; q += 32) s = fma(m[q], rv[q], s);
                s = warp_sum(s);
                if (lane == 0) {
                    int k = row % (Z + 1), j = (row / (Z + 1)) % (Y + 1), i = row / ((Z + 1) * (Y + 1));
                    P[L][(i + 1) * sx + (j + 1) * sy + (k + 1)] = s;
                }
            }
            __syncthreads();
        } else {
            __syncthreads();
            if (tid < 32) coarse_rbgs_warp(P[L], R[L], bc.E[0], bc.E[1], bc.E[2], a.kkc, bc, a.tol, a.maxc, a.iters);
            __syncthreads();
        }
    }
    // back up: prolongation + add, post-smoothing
    for (int l = a.nl - 2; l >= 0; --l) {
        const MgBC &bc = a.bc[l], &bcc = a.bc[l + 1];
        int E1 = bc.E[1], E2 = bc.E[2], sy = E2 + 3, sx = (E1 + 3) * sy;
        T *pf = P[l];
        View3<const T> C; C.p = P[l + 1]; C.sy = bcc.E[2] + 3; C.sx = (bcc.E[1] + 3) * C.sy;
        tail_for(bc.E[0] + 1, E1 + 1, E2 + 1, [&](int i, int j, int k) {
            int i2 = i / 2, j2 = j / 2, k2 = k / 2;
            bool io = i & 1, jo = j & 1, ko = k & 1;
            T v;
            if (io) {
                if (jo) {
                    if (ko) v = (C(i2, j2, k2) + C(i2 + 1, j2, k2) + C(i2, j2 + 1, k2) + C(i2, j2, k2 + 1) + C(i2 + 1, j2 + 1, k2) +
                                 C(i2 + 1, j2, k2 + 1) + C(i2, j2 + 1, k2 + 1) + C(i2 + 1, j2 + 1, k2 + 1)) * (T)0.125;
                    else v = (C(i2, j2, k2) + C(i2, j2 + 1, k2) + C(i2 + 1, j2, k2) + C(i2 + 1, j2 + 1, k2)) * (T)0.25;
                } else {
                    if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1) + C(i2 + 1, j2, k2) + C(i2 + 1, j2, k2 + 1)) * (T)0.25;
                    else v = (C(i2, j2, k2) + C(i2 + 1, j2, k2)) * (T)0.5;
                }
            } else {
                if (jo) {
                    if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1) + C(i2, j2 + 1, k2) + C(i2, j2 + 1, k2 + 1)) * (T)0.25;
                    else v = (C(i2, j2, k2) + C(i2, j2 + 1, k2)) * (T)0.5;
                } else {
                    if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1)) * (T)0.5;
                    else v = C(i2, j2, k2);
                }
            }
            int o = (i + 1) * sx + (j + 1) * sy + (k + 1);
            v = v + pf[o];
            pf[o] = v;
            if (near_face<T>(i, j, k, bc)) tgt_images(pf, sx, sy, i, j, k, v, bc);
        });
        __syncthreads();
        for (int m = 0; m < a.post; ++m) {
            tail_sweep<T, false>(Q[l], P[l], R[l], bc, tgk_weight(a.tk[l], a.wpost[m]));
            T *x = P[l]; P[l] = Q[l]; Q[l] = x;
        }
    }
    for (int t = tid; t < tail_count<T>(a.bc[0]); t += nt) a.pout[t] = P[0][t];
}

// ------------------------------------------------------------------ host
static MgBC level_bc(const Ctx &c, int l, bool tgt) {
    MgBC b;
    b.per[0] = c.p.xPer; b.per[1] = c.planar ? 0 : c.p.yPer; b.per[2] = c.p.zPer;
    for (int d = 0; d < 3; ++d) b.E[d] = c.lv[l].n[d];
    b.planar = c.planar ? 1 : 0;
    b.dirichlet = c.p.testPoisson && !tgt;
    b.zeroBC = (l != 0);
    b.tgtPads = tgt ? 1 : 0;
    return b;
}

template <typename T>
static View3<T> lview(const Level &L, T *p) { return make_view<T>(p, L.n[0] + 1, L.n[1] + 1, L.n[2] + 1); }
template <typename T>
static View3<const T> lcview(const Level &L, const T *p) {
    View3<T> w = make_view<T>(const_cast<T *>(p), L.n[0] + 1, L.n[1] + 1, L.n[2] + 1);
    View3<const T> v; v.p = w.p; v.n[0] = w.n[0]; v.n[1] = w.n[1]; v.n[2] = w.n[2]; v.sx = w.sx; v.sy = w.sy;
    return v;
}

static void core_dims(const Level &L, dim3 &g, dim3 &b) {
    int nz = L.n[2] + 1, ny = L.n[1] + 1, nx = L.n[0] + 1;
    b = nz >= 64 ? dim3(64, 4, 1) : nz >= 32 ? dim3(32, 8, 1) : dim3(16, 8, 2);
    g = dim3((nz + b.x - 1) / b.x, (ny + b.y - 1) / b.y, (nx + b.z - 1) / b.z);
}

static int chk(Ctx &c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { c.err = std::string(what) + ": " + cudaGetErrorString(e); return SARAS_CUDA_ERROR; }
    return SARAS_OK;
}

// First level of the fused coarse tail (k_mg_tail), or -1: all axes at most 16
// intervals, at least two levels, and every tail level in shared memory.
static int tail_level(const Ctx &c) {
    if (c.p.preSmooth > kTailMaxSweeps || c.p.postSmooth > kTailMaxSweeps || c.p.coarseSmooth > kTailMaxSweeps) return -1;
    for (int l = 1; l < c.depth; ++l) {
        const Level &L = c.lv[l];
        if (std::max(L.n[0], std::max(L.n[1], L.n[2])) > kTailIntervals) continue;
        if (c.depth - l + 1 > kTailMaxLevels) return -1;
        size_t bytes = 0;
        for (int q = l; q <= c.depth; ++q) bytes += 3 * sizeof(double) * (size_t)c.lv[q].count;
        return bytes <= 200 * 1024 ? l : -1;
    }
    return -1;
}

// Solution operator of the coarsest level of the fused tail.  The target-mode
// coarsest problem A e = r (the level Laplacian with mirror / periodic ghosts)
// is singular: A 1 = 0 and w^T A = 0 for the trapezoidal weights w.  M is the
// top-left n x n block of the inverse of the bordered matrix [[A, 1], [w^T, 0]],
// so e = M r solves A e = r - (w.r / w.1) 1 with w.e = 0: the compatible
// system that the Gauss-Seidel path solves after removing the weighted mean,
// here exactly.  Points are numbered k fastest, then j, then i.  Gauss-Jordan
// elimination with partial pivoting in FP64; false if a pivot vanishes.
static bool coarse_solution_operator(int X, int Y, int Z, const double l[3], const int per[3], std::vector<double> &M) {
    const int E[3] = {X, Y, Z};
    const int n = (X + 1) * (Y + 1) * (Z + 1), N = n + 1;
    auto id = [&](const int q[3]) { return (q[0] * (Y + 1) + q[1]) * (Z + 1) + q[2]; };
    auto img = [&](int q, int d) { return q < 0 ? (per[d] ? E[d] - 1 : 1) : q > E[d] ? (per[d] ? 1 : E[d] - 1) : q; };
    std::vector<double> B((size_t)N * N, 0.0), R((size_t)N * n, 0.0);
    int q[3];
    for (q[0] = 0; q[0] <= X; ++q[0])
        for (q[1] = 0; q[1] <= Y; ++q[1])
            for (q[2] = 0; q[2] <= Z; ++q[2]) {
                int P = id(q);
                double w = 1.0;
                for (int d = 0; d < 3; ++d) {
                    B[(size_t)P * N + P] -= 2.0 * l[d];
                    for (int s = -1; s <= 1; s += 2) {
                        int r[3] = {q[0], q[1], q[2]};
                        r[d] = img(q[d] + s, d);
                        B[(size_t)P * N + id(r)] += l[d];
                    }
                    if (q[d] == 0 || q[d] == E[d]) w *= 0.5;
                }
                B[(size_t)P * N + n] = 1.0;
                B[(size_t)n * N + P] = w;
                R[(size_t)P * n + P] = 1.0;
            }
    for (int col = 0; col < N; ++col) {
        int piv = col;
        for (int r = col + 1; r < N; ++r)
            if (std::fabs(B[(size_t)r * N + col]) > std::fabs(B[(size_t)piv * N + col])) piv = r;
        if (!(std::fabs(B[(size_t)piv * N + col]) > 1e-300)) return false;
        if (piv != col) {
            for (int t = 0; t < N; ++t) std::swap(B[(size_t)piv * N + t], B[(size_t)col * N + t]);
            for (int t = 0; t < n; ++t) std::swap(R[(size_t)piv * n + t], R[(size_t)col * n + t]);
        }
        double inv = 1.0 / B[(size_t)col * N + col];
        for (int t = 0; t < N; ++t) B[(size_t)col * N + t] *= inv;
        for (int t = 0; t < n; ++t) R[(size_t)col * n + t] *= inv;
        for (int r = 0; r < N; ++r) {
            if (r == col) continue;
            double f = B[(size_t)r * N + col];
            if (f == 0.0) continue;
            for (int t = 0; t < N; ++t) B[(size_t)r * N + t] -= f * B[(size_t)col * N + t];
            for (int t = 0; t < n; ++t) R[(size_t)r * n + t] -= f * R[(size_t)col * n + t];
        }
    }
    M.assign(R.begin(), R.begin() + (size_t)n * n);
    return true;
}

// Tensor maps and launch shape of the finest-level plane-streaming kernels
// (k_tgt_plane_tma).  The level array is viewed as rows of kPlaneVec floats;
// the main box covers a tile's rows j0-1 .. j0+R of a plane, the side box one
// padded row, the right-hand side's box rows j0 .. j0+R-1.  Used when
// SARAS_PLANE_TMA=1 is set in the environment and the level fits (at least
// two tiles of rows, the ring within 200 KB); otherwise the column kernels run.
// Both compute the same bits; the column kernels are the default because they
// are faster on GB300 (257^3 level-0 sweep: 0.046 ms against 0.071 ms).
// The driver's cuTensorMapEncodeTiled, looked up through the runtime (the
// library does not link the driver library, so it loads on machines without
// one and reports SARAS_NO_DEVICE there).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

static int plane_setup(Ctx &c) {
    c.planeOk = false;
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return SARAS_OK;
    const char *env = std::getenv("SARAS_PLANE_TMA");
    if (!env || env[0] != '1') return SARAS_OK;
    Level &L = c.lv[0];
    const int E0 = L.n[0], E1 = L.n[1], E2 = L.n[2];
    const int sy = E2 + 3, W = E2 + 1;
    const int nTiles = (E1 + 1) / kPlaneRows;
    if (nTiles < 2 || E0 < 2) return SARAS_OK;
    const int maxRows = (E1 + 1) - kPlaneRows * (nTiles - 1);
    const int maxq = (maxRows * W + kPlaneThreads - 1) / kPlaneThreads;
    if (maxq > 11) return SARAS_OK;
    // box heights in rows of kPlaneVec floats: a span plus up to kPlaneVec - 1
    // floats before its start (the copy starts at the boundary below it).
    // TMA writes shared memory at 128-byte aligned addresses: every box starts
    // at a multiple of kPlaneVec floats in its slot
    const long mainRows = ((long)(maxRows + 2) * sy + 2 * kPlaneVec - 2) / kPlaneVec;
    const long sideRows = ((long)sy + 2 * kPlaneVec - 2) / kPlaneVec;
    const long rRows = ((long)maxRows * sy + 2 * kPlaneVec - 2) / kPlaneVec;
    if (mainRows > 256 || sideRows > 256 || rRows > 256) return SARAS_OK;
    const int sideOff = (int)mainRows * kPlaneVec, rOff = sideOff + (int)sideRows * kPlaneVec;
    const int slot = rOff + (int)rRows * kPlaneVec;
    const size_t smem = (size_t)kPlaneRing * slot * sizeof(float) + 128;   // + alignment of the first slot
    if (smem > 200 * 1024) return SARAS_OK;
    cuuint64_t dims[2] = {(cuuint64_t)kPlaneVec, (cuuint64_t)(L.count / kPlaneVec)};
    cuuint64_t strides[1] = {(cuuint64_t)kPlaneVec * sizeof(float)};
    cuuint32_t box[2] = {(cuuint32_t)kPlaneVec, (cuuint32_t)mainRows}, sbox[2] = {(cuuint32_t)kPlaneVec, (cuuint32_t)sideRows},
               rbox[2] = {(cuuint32_t)kPlaneVec, (cuuint32_t)rRows};
    cuuint32_t es[2] = {1, 1};
    auto enc = [&](CUtensorMap *m, float *base, const cuuint32_t *bx) {
        return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    };
    for (int b = 0; b < 2; ++b) {
        float *base = b ? L.b32 : L.a32;
        if (!enc(&c.planeMap[b], base, box) || !enc(&c.planeSide[b], base, sbox)) return SARAS_OK;   // the other kernels run
    }
    if (!enc(&c.planeR, L.r32, rbox)) return SARAS_OK;
    c.planeMaxQ = maxq <= 5 ? 5 : 11;
    const void *fns[2] = {c.planeMaxQ == 5 ? (const void *)k_tgt_plane_tma<0, 5> : (const void *)k_tgt_plane_tma<0, 11>,
                          c.planeMaxQ == 5 ? (const void *)k_tgt_plane_tma<1, 5> : (const void *)k_tgt_plane_tma<1, 11>};
    for (const void *f : fns) SARAS_CUDA_TRY(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // one wave: as many CTAs as fit (shared memory bounds them), tiles x segments of planes
    int perSM = 0;
    SARAS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fns[0], kPlaneThreads, smem));
    perSM = std::max(1, perSM);
    const int segs0 = std::max(1, (c.numSMs * perSM) / nTiles);
    c.planeSegPlanes = (E0 + 1 + segs0 - 1) / segs0;
    c.planeSegs = (E0 + 1 + c.planeSegPlanes - 1) / c.planeSegPlanes;
    c.planeMainRows = (int)mainRows;
    c.planeSideRows = (int)sideRows;
    c.planeRRows = (int)rRows;
    c.planeSideOff = sideOff;
    c.planeROff = rOff;
    c.planeSlotFloats = slot;
    c.planeSmem = smem;
    c.planeOk = true;
    return SARAS_OK;
}

// Finest-level FP32 sweep (mode 0) or residual (mode 1) through the plane-streaming kernel.
static void plane_launch(Ctx &c, int mode, float *out, const float *in, const float *r, const MgBC &bc, const TgK<float> &tk) {
    Level &L = c.lv[0];
    (void)r;   // the right-hand side comes through its tensor map (the level's r32)
    PlaneArgs a;
    a.out = out;
    a.sy = L.n[2] + 3;
    a.sx = (L.n[1] + 3) * a.sy;
    a.bc = bc;
    a.c = tk;
    a.mainRows = c.planeMainRows;
    a.sideRows = c.planeSideRows;
    a.rRows = c.planeRRows;
    a.sideOff = c.planeSideOff;
    a.rOff = c.planeROff;
    a.slotFloats = c.planeSlotFloats;
    a.planesPerSeg = c.planeSegPlanes;
    a.err = c.dflag + 2;
    const int b = in == L.a32 ? 0 : 1;
    dim3 g((L.n[1] + 1) / kPlaneRows, c.planeSegs, 1);
    if (c.planeMaxQ == 5) {
        if (mode == 0) k_tgt_plane_tma<0, 5><<<g, kPlaneThreads, c.planeSmem, c.stream>>>(c.planeMap[b], c.planeSide[b], c.planeR, a);
        else k_tgt_plane_tma<1, 5><<<g, kPlaneThreads, c.planeSmem, c.stream>>>(c.planeMap[b], c.planeSide[b], c.planeR, a);
    } else {
        if (mode == 0) k_tgt_plane_tma<0, 11><<<g, kPlaneThreads, c.planeSmem, c.stream>>>(c.planeMap[b], c.planeSide[b], c.planeR, a);
        else k_tgt_plane_tma<1, 11><<<g, kPlaneThreads, c.planeSmem, c.stream>>>(c.planeMap[b], c.planeSide[b], c.planeR, a);
    }
}

int mg_setup(Ctx &c) {
    const saras_params &p = c.p;
    c.depth = p.vcDepth;
    c.mgMode = p.mgMode;
    c.mgTarget = p.mgTarget;
    c.mgMaxCycles = p.mgMaxCycles;
    int ind[3] = {p.xInd, p.yInd, p.zInd};
    c.lv.assign(c.depth + 1, Level());
    for (int l = 0; l <= c.depth; ++l) {
        Level &L = c.lv[l];
        for (int d = 0; d < 3; ++d) L.n[d] = int(std::pow(2, ind[d] - l));          // poisson.cc:336-357
        if (c.planar) L.n[1] = 0;                                                      // poisson.cc:339-340: one y point
        L.count = (long)(L.n[0] + 3) * (L.n[1] + 3) * (L.n[2] + 3);
        double s = std::pow(2, l);
        double dXi = c.dXi[0], dEt = c.dXi[1], dZt = c.dXi[2];
        L.hx = s * dXi; L.hy = s * dEt; L.hz = s * dZt;                                  // poisson.cc:419-438
        L.hxhy = std::pow(s, 4.0) * std::pow(dXi, 2.0) * std::pow(dEt, 2.0);
        L.hyhz = std::pow(s, 4.0) * std::pow(dEt, 2.0) * std::pow(dZt, 2.0);
        L.hzhx = std::pow(s, 4.0) * std::pow(dZt, 2.0) * std::pow(dXi, 2.0);
        L.hxhyhz = std::pow(s, 6.0) * std::pow(dXi, 2.0) * std::pow(dEt, 2.0) * std::pow(dZt, 2.0);
        double xix2 = c.m2[0], ety2 = c.m2[1], ztz2 = c.m2[2];                            // poisson.cc:463-495
        L.cx = L.hyhz * xix2; L.cy = L.hzhx * ety2; L.cz = L.hxhy * ztz2;
        L.c7 = 2.0 * L.hxhyhz;
        L.den = 4.0 * (L.hyhz * xix2 + L.hzhx * ety2 + L.hxhy * ztz2);
        L.ihx2 = 1.0 / (L.hx * L.hx); L.ihy2 = 1.0 / (L.hy * L.hy); L.ihz2 = 1.0 / (L.hz * L.hz);
        L.lx = xix2 * L.ihx2; L.ly = ety2 * L.ihy2; L.lz = ztz2 * L.ihz2;
        L.hx2 = std::pow(s * dXi, 2.0); L.hz2 = std::pow(s * dZt, 2.0);
        L.planar = c.planar ? 1 : 0;
        if (c.stretched || c.planar) {   // the stencils read the metrics at each point
            // poisson.cc:463-495: the staggered metrics of the finest grid at every
            // 2^l-th point on the level's core, 0 at its two ghost indices
            const int s2 = 1 << l;
            const size_t len[3] = {(size_t)L.n[0] + 3, (size_t)L.n[1] + 3, (size_t)L.n[2] + 3};
            std::vector<double> h(2 * (len[0] + len[1] + len[2]), 0.0);
            size_t off[6];
            size_t o = 0;
            for (int d = 0; d < 3; ++d)
                for (int m = 0; m < 2; ++m) {   // m 0: xix2, 1: xixx
                    off[2 * d + m] = o;
                    const std::vector<double> &src = c.hmet[d][1][m == 0 ? 2 : 1];
                    for (int i = 0; i <= L.n[d]; ++i) h[o + 1 + i] = src[(size_t)i * s2 + 1];
                    o += len[d];
                }
            SARAS_CUDA_TRY(cudaMalloc(&L.metBlock, sizeof(double) * h.size()));
            SARAS_CUDA_TRY(cudaMemcpy(L.metBlock, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
            L.xix2 = L.metBlock + off[0] + 1; L.xixx = L.metBlock + off[1] + 1;
            L.ety2 = L.metBlock + off[2] + 1; L.etyy = L.metBlock + off[3] + 1;
            L.ztz2 = L.metBlock + off[4] + 1; L.ztzz = L.metBlock + off[5] + 1;
        }
        size_t b64 = sizeof(double) * L.count, b32 = sizeof(float) * L.count;
        SARAS_CUDA_TRY(cudaMalloc(&L.a, b64)); SARAS_CUDA_TRY(cudaMalloc(&L.b, b64)); SARAS_CUDA_TRY(cudaMalloc(&L.r, b64));
        SARAS_CUDA_TRY(cudaMemsetAsync(L.a, 0, b64, c.stream)); SARAS_CUDA_TRY(cudaMemsetAsync(L.b, 0, b64, c.stream));
        SARAS_CUDA_TRY(cudaMemsetAsync(L.r, 0, b64, c.stream));
        SARAS_CUDA_TRY(cudaMalloc(&L.a32, b32)); SARAS_CUDA_TRY(cudaMalloc(&L.b32, b32)); SARAS_CUDA_TRY(cudaMalloc(&L.r32, b32));
        SARAS_CUDA_TRY(cudaMemsetAsync(L.a32, 0, b32, c.stream)); SARAS_CUDA_TRY(cudaMemsetAsync(L.b32, 0, b32, c.stream));
        SARAS_CUDA_TRY(cudaMemsetAsync(L.r32, 0, b32, c.stream));
    }
    const Level &C = c.lv[c.depth];
    c.maxCount = (C.n[0] + 2) * (C.n[1] + 2) * (C.n[2] + 2);                            // poisson.cc:360-361
    size_t smem = 2 * sizeof(double) * C.count;
    if (smem > 220 * 1024) { c.err = "coarsest multigrid level too large for one CTA; increase V-Cycle Depth"; return SARAS_BAD_CONFIG; }
    SARAS_CUDA_TRY(cudaFuncSetAttribute(k_mg_coarse<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SARAS_CUDA_TRY(cudaFuncSetAttribute(k_mg_coarse<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SARAS_CUDA_TRY(cudaDeviceGetAttribute(&c.numSMs, cudaDevAttrMultiProcessorCount, c.dev));
    SARAS_CUDA_TRY(cudaFuncSetAttribute(k_mg_gs_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGsBlockSmem));
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dflag, 0, 3 * sizeof(int), c.stream));
    if (int e = plane_setup(c)) return e;
    c.tailLt = c.planar ? 0 : tail_level(c);   // target modes only (3D)
    if (c.tailLt > 0) {
        SARAS_CUDA_TRY(cudaFuncSetAttribute(k_mg_tail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        SARAS_CUDA_TRY(cudaFuncSetAttribute(k_mg_tail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        // the tail's coarsest solve as a matrix-vector product when the level is small
        const Level &Lc = c.lv[c.depth];
        long nc = (long)(Lc.n[0] + 1) * (Lc.n[1] + 1) * (Lc.n[2] + 1);
        double l[3] = {Lc.lx, Lc.ly, Lc.lz};
        int per[3] = {p.xPer, p.yPer, p.zPer};
        std::vector<double> M;
        if (nc <= 512 && coarse_solution_operator(Lc.n[0], Lc.n[1], Lc.n[2], l, per, M)) {
            std::vector<float> M32(M.begin(), M.end());
            SARAS_CUDA_TRY(cudaMalloc(&c.coarseM64, M.size() * sizeof(double)));
            SARAS_CUDA_TRY(cudaMalloc(&c.coarseM32, M32.size() * sizeof(float)));
            SARAS_CUDA_TRY(cudaMemcpy(c.coarseM64, M.data(), M.size() * sizeof(double), cudaMemcpyHostToDevice));
            SARAS_CUDA_TRY(cudaMemcpy(c.coarseM32, M32.data(), M32.size() * sizeof(float), cudaMemcpyHostToDevice));
            c.coarseN = (int)nc;
        }
    }
    if (p.testPoisson) {
        // multigrid_d3::initDirichlet (poisson_d3.cc:513-572), np = 1
        const Level &L0 = c.lv[0];
        int X = L0.n[0], Y = L0.n[1], Z = L0.n[2];
        std::vector<double> wx((size_t)(Y + 3) * (Z + 3), 0.0), wy((size_t)(X + 3) * (Z + 3), 0.0), wz((size_t)(X + 3) * (Y + 3), 0.0);
        int hX = X / 2, hY = Y / 2;
        double xd, yd, zd;
        xd = L0.hx + p.Lx / 2.0;
        for (int j = 0; j <= Y; ++j) { yd = L0.hy * (j - hY); for (int k = 0; k <= Z; ++k) { zd = L0.hz * (k - Z / 2); wx[(j + 1) * (Z + 3) + k + 1] = (xd * xd + yd * yd + zd * zd) / 6.0; } }
        yd = L0.hy + p.Ly / 2.0;
        for (int i = 0; i <= X; ++i) { xd = L0.hx * (i - hX); for (int k = 0; k <= Z; ++k) { zd = L0.hz * (k - Z / 2); wy[(i + 1) * (Z + 3) + k + 1] = (xd * xd + yd * yd + zd * zd) / 6.0; } }
        zd = L0.hz + p.Lz / 2.0;
        for (int i = 0; i <= X; ++i) { xd = L0.hx * (i - hX); for (int j = 0; j <= Y; ++j) { yd = L0.hy * (j - hY); wz[(i + 1) * (Y + 3) + j + 1] = (xd * xd + yd * yd + zd * zd) / 6.0; } }
        SARAS_CUDA_TRY(cudaMalloc(&c.wallX, wx.size() * 8)); SARAS_CUDA_TRY(cudaMalloc(&c.wallY, wy.size() * 8)); SARAS_CUDA_TRY(cudaMalloc(&c.wallZ, wz.size() * 8));
        SARAS_CUDA_TRY(cudaMemcpy(c.wallX, wx.data(), wx.size() * 8, cudaMemcpyHostToDevice));
        SARAS_CUDA_TRY(cudaMemcpy(c.wallY, wy.data(), wy.size() * 8, cudaMemcpyHostToDevice));
        SARAS_CUDA_TRY(cudaMemcpy(c.wallZ, wz.data(), wz.size() * 8, cudaMemcpyHostToDevice));
    }
    return SARAS_OK;
}

void mg_free(Ctx &c) {
    vgraph_reset(c);
    for (Level &L : c.lv) {
        cudaFree(L.a); cudaFree(L.b); cudaFree(L.r); cudaFree(L.a32); cudaFree(L.b32); cudaFree(L.r32); cudaFree(L.metBlock);
    }
    for (long long *&q : c.fx) { cudaFree(q); q = nullptr; }
    c.lv.clear();
    cudaFree(c.wallX); cudaFree(c.wallY); cudaFree(c.wallZ);
    c.wallX = c.wallY = c.wallZ = nullptr;
    cudaFree(c.coarseM64); cudaFree(c.coarseM32);
    c.coarseM64 = nullptr; c.coarseM32 = nullptr; c.coarseN = 0;
}

// Level-0 Dirichlet wall values into the face ghosts of a level-0 array
// (zeroBC = false at level 0; constant for the whole solve).
__global__ void k_dirichlet_walls(View3<double> p, MgBC bc, const double *wx, const double *wy, const double *wz) {
    int i, j, k;
    int E[3] = {bc.E[0] + 2, bc.E[1] + 2, bc.E[2] + 2};
    if (!core_pt(E, i, j, k)) return;
    i -= 1; j -= 1; k -= 1;
    int gi = (i < 0 || i > bc.E[0]), gj = (j < 0 || j > bc.E[1]), gk = (k < 0 || k > bc.E[2]);
    if (gi + gj + gk != 1) return;
    if (gi) p(i, j, k) = wx[(j + 1) * (bc.E[2] + 3) + k + 1];
    if (gj) p(i, j, k) = wy[(i + 1) * (bc.E[2] + 3) + k + 1];
    if (gk) p(i, j, k) = wz[(i + 1) * (bc.E[1] + 3) + j + 1];
}

// ---- generic level operations (templated on precision)
template <typename T> static T *A_(Level &L);
template <> double *A_<double>(Level &L) { return L.pa(); }
template <> float *A_<float>(Level &L) { return L.pa32(); }
template <typename T> static T *B_(Level &L);
template <> double *B_<double>(Level &L) { return L.pb(); }
template <> float *B_<float>(Level &L) { return L.pb32(); }
template <typename T> static T *R_(Level &L);
template <> double *R_<double>(Level &L) { return L.r; }
template <> float *R_<float>(Level &L) { return L.r32; }
template <typename T> static void flip(Level &L);
template <> void flip<double>(Level &L) { L.cur ^= 1; }
template <> void flip<float>(Level &L) { L.cur32 ^= 1; }

// Weight of sweep n of a target-mode smoothing phase of `count` sweeps.
// Damped Jacobi: jacobiWeight throughout.  Chebyshev (smoother = 1): the phase
// is the degree-count Chebyshev polynomial of D^-1 A (its spectrum is in
// [0, 2] for the mirror / periodic 7-point Laplacian) that is smallest on the
// modes the coarse grid cannot represent, lambda in [1/3, 2]: sweep n has the
// weight 1 / lambda_n for a root lambda_n of that polynomial.  The roots are
// taken alternately from the two ends of the interval, which keeps the
// intermediate iterates' growth small.  For 4 sweeps the polynomial is below
// 0.062 on [1/3, 2]; damped Jacobi with weight 6/7 gives (5/7)^4 = 0.26.
static double smooth_weight(const Ctx &c, int n, int count) {
    if (c.p.smoother != 1 || count < 1) return c.p.jacobiWeight;
    const double a = 1.0 / 3.0, b = 2.0;
    int r = (n % 2 == 0) ? n / 2 : count - 1 - n / 2;   // 0, m-1, 1, m-2, ...
    double lam = 0.5 * (b + a) + 0.5 * (b - a) * std::cos(M_PI * (2.0 * r + 1.0) / (2.0 * count));
    return 1.0 / lam;
}

// Gauss-Seidel smoothing of level l (reference mode with gsSmooth = 1): one
// CTA from shared memory for levels up to kGsBlockSmem of iterate plus
// right-hand side, else the cooperative grid kernel with one block an SM at
// most (a stage has at most (X+1)(Y+1) points).
static int gs_smooth(Ctx &c, int l, int count, bool zero_first) {
    Level &L = c.lv[l];
    MgBC bc = level_bc(c, l, false);
    MgK kk = make_k(L);
    const bool walls = bc.dirichlet && !bc.zeroBC;
    const double *wx = walls ? c.wallX : nullptr, *wy = walls ? c.wallY : nullptr, *wz = walls ? c.wallZ : nullptr;
    View3<double> pv = lview<double>(L, L.pa());
    View3<const double> rv = lcview<double>(L, L.r);
    const size_t smem = 2 * sizeof(double) * (size_t)L.count;
    if (smem <= kGsBlockSmem) {
        k_mg_gs_block<<<1, 512, smem, c.stream>>>(pv, rv, kk, bc, count, zero_first ? 1 : 0, wx, wy, wz);
        count_launch(c);
        return chk(c, "mg Gauss-Seidel");
    }
    if (zero_first) SARAS_CUDA_TRY(cudaMemsetAsync(L.pa(), 0, sizeof(double) * (size_t)L.count, c.stream));
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dflag, 0, sizeof(int), c.stream));   // barrier arrivals
    const long pairs = (long)(L.n[0] + 1) * (L.n[1] + 1);
    int blocks = (int)std::max<long>(1, std::min<long>((pairs + 255) / 256, c.numSMs));
    unsigned *sync = reinterpret_cast<unsigned *>(c.dflag);
    int *err = c.dflag + 1;
    void *args[] = {&pv, &rv, &kk, &bc, &count, &sync, &err, &wx, &wy, &wz};
    SARAS_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_mg_gs_grid, dim3(blocks), dim3(256), args, 0, c.stream));
    count_launch(c);
    return chk(c, "mg Gauss-Seidel");
}

// Status of the Gauss-Seidel grid barriers since the last reset (synchronises).
static int gs_status(Ctx &c) {
    int e = 0;
    SARAS_CUDA_TRY(cudaMemcpyAsync(&e, c.dflag + 1, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (e) { c.err = "Gauss-Seidel smoothing: a grid barrier wait timed out"; return SARAS_CUDA_ERROR; }
    return SARAS_OK;
}

template <typename T>
static int smooth(Ctx &c, int l, int count, bool zero_first, bool tgt) {
    if (!tgt && c.p.gsSmooth && sizeof(T) == 8) return gs_smooth(c, l, count, zero_first);
    Level &L = c.lv[l];
    MgBC bc = level_bc(c, l, tgt);
    MgK kk = make_k(L);
    dim3 g, b; core_dims(L, g, b);
    T omega = tgt ? (T)c.p.jacobiWeight : (T)1.0;
    int pk = sizeof(T) == 8 ? PK_MG_SMOOTH64 : PK_MG_SMOOTH32;
    double bytes = 3.0 * sizeof(T) * (double)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1);
    int sx = (L.n[1] + 3) * (L.n[2] + 3), sy = L.n[2] + 3;
    dim3 gm, bm; level_dims<T>(L, gm, bm);
    for (int n = 0; n < count; ++n) {
        TgK<T> tk = make_tgk<T>(L, tgt ? smooth_weight(c, n, count) : c.p.jacobiWeight);
        prof_begin(c, pk, l);
        const double lb = (n == 0 && zero_first) ? bytes * 2.0 / 3.0 : bytes;   // a zero start reads no iterate
        if (tgt) {
            if constexpr (sizeof(T) == 4) {
                if (n == 0 && zero_first && count >= 2 && !(l == 0 && c.planeOk)) {
                    // sweeps 0 and 1 in one launch, written where the second would leave
                    // the iterate (the current buffer: two flips), so no flip
                    TgK<T> tk2 = make_tgk<T>(L, smooth_weight(c, 1, count));
                    SARAS_CUDA_TRY(launch_pdl(k_tgt_sweep2z<T>, gm, bm, 0, c.stream, A_<T>(L), R_<T>(L), sx, sy, bc, tk, tk2));
                    count_launch(c);
                    prof_end(c, pk, l, lb);
                    ++n;
                    continue;
                }
            }
            if (n == 0 && zero_first) SARAS_CUDA_TRY(launch_pdl(k_tgt_sweep<T, true>, gm, bm, 0, c.stream, B_<T>(L), A_<T>(L), R_<T>(L), sx, sy, bc, tk));
            else if constexpr (sizeof(T) == 4) {
                if (l == 0 && c.planeOk) plane_launch(c, 0, B_<T>(L), A_<T>(L), R_<T>(L), bc, tk);
                else SARAS_CUDA_TRY(launch_pdl(k_tgt_sweep<T, false>, gm, bm, 0, c.stream, B_<T>(L), A_<T>(L), R_<T>(L), sx, sy, bc, tk));
            } else SARAS_CUDA_TRY(launch_pdl(k_tgt_sweep<T, false>, gm, bm, 0, c.stream, B_<T>(L), A_<T>(L), R_<T>(L), sx, sy, bc, tk));
        } else if (n == 0 && zero_first)
            k_mg_sweep<T, true><<<g, b, 0, c.stream>>>(lview<T>(L, B_<T>(L)), lcview<T>(L, A_<T>(L)), lcview<T>(L, R_<T>(L)), kk, bc, omega);
        else
            k_mg_sweep<T, false><<<g, b, 0, c.stream>>>(lview<T>(L, B_<T>(L)), lcview<T>(L, A_<T>(L)), lcview<T>(L, R_<T>(L)), kk, bc, omega);
        count_launch(c);
        prof_end(c, pk, l, lb);
        flip<T>(L);
    }
    return chk(c, "mg smooth");
}

// Threads of the single-CTA coarsest Gauss-Seidel solve.  Its wavefront stages
// hold at most (X + 1)(Y + 1) points (25 on a 5^3 level, one warp); the residual
// check after each sweep takes the whole level.  Measured on the 33^3 cavity
// (217 sweeps a V-cycle on the 5^3 level): 2.91 ms a V-cycle with 128 threads,
// 2.98 with 64, 3.03 with 256, 3.26 with 32.  Slower, and not kept: a stage's
// points dealt across the warps instead of packed into one (3.04); the residual
// check formed inside the sweep, plane s - 2 by the block's second half during
// stage s (3.20: the two halves share the SM's FP64 pipe).
constexpr int kCoarseThreads = 128;

template <typename T>
static int coarse_solve(Ctx &c, bool tgt) {
    Level &L = c.lv[c.depth];
    MgBC bc = level_bc(c, c.depth, tgt);
    MgK kk = make_k(L);
    size_t smem = 2 * sizeof(T) * L.count;
    // target modes: the coarsest correction only has to be small against the
    // V-cycle's own error reduction (about 0.1), so 1e-3 of the initial residual
    T tol = tgt ? (T)1.0e-3 : (T)c.p.mgTolerance;
    int maxc = tgt ? 500 : c.maxCount;
    k_mg_coarse<T><<<1, kCoarseThreads, smem, c.stream>>>(lview<T>(L, A_<T>(L)), lcview<T>(L, R_<T>(L)), kk, bc, tol, maxc, tgt ? 1 : 0,
                                               (long long *)(c.dscal + 40));
    count_launch(c);
    return chk(c, "mg coarse");
}

template <typename T>
static int restrict_level(Ctx &c, int l, bool tgt) {
    Level &L = c.lv[l], &C = c.lv[l + 1];
    MgBC bcf = level_bc(c, l, tgt), bcc = level_bc(c, l + 1, tgt);
    MgK kk = make_k(L);
    dim3 g, b; core_dims(L, g, b);
    int pk = sizeof(T) == 8 ? PK_MG_RESID64 : PK_MG_RESID32;
    double pts = (double)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1);
    prof_begin(c, pk, l);
    if (tgt) {
        int sx = (L.n[1] + 3) * (L.n[2] + 3), sy = L.n[2] + 3;
        dim3 gm, bm; level_dims<T>(L, gm, bm);
        bool planed = false;
        if constexpr (sizeof(T) == 4) {
            if (l == 0 && c.planeOk) {
                plane_launch(c, 1, B_<T>(L), A_<T>(L), R_<T>(L), bcf, make_tgk<T>(L, 1.0));
                planed = true;
            }
        }
        if (!planed)
            SARAS_CUDA_TRY(launch_pdl(k_tgt_residual<T, T, false>, gm, bm, 0, c.stream, B_<T>(L), A_<T>(L), R_<T>(L), sx, sy, bcf,
                                      make_tgk<T>(L, 1.0), (double *)nullptr));
        count_launch(c);
        prof_end(c, pk, l, 3.0 * sizeof(T) * pts);
        pk = sizeof(T) == 8 ? PK_MG_RESTRICT64 : PK_MG_RESTRICT32;
        prof_begin(c, pk, l);
        int csx = (C.n[1] + 3) * (C.n[2] + 3), csy = C.n[2] + 3;
        long ccols = (long)(C.n[1] + 1) * (C.n[2] + 1);
        dim3 gr((unsigned)((ccols + 255) / 256), (C.n[0] + 1 + rr_ch<T>() - 1) / rr_ch<T>(), 1);
        SARAS_CUDA_TRY(launch_pdl(k_tgt_restrict<T>, gr, dim3(256, 1, 1), 0, c.stream, R_<T>(C), B_<T>(L), sx, sy, csx, csy, bcf));
        count_launch(c);
        prof_end(c, pk, l, sizeof(T) * pts * (1.0 + 1.0 / 8.0));
        return chk(c, "mg restrict");
    } else
        k_mg_residual<T><<<g, b, 0, c.stream>>>(lview<T>(L, B_<T>(L)), lcview<T>(L, A_<T>(L)), lcview<T>(L, R_<T>(L)), kk, bcf);
    count_launch(c);
    prof_end(c, pk, l, 3.0 * sizeof(T) * pts);
    dim3 g2, b2; core_dims(C, g2, b2);
    pk = sizeof(T) == 8 ? PK_MG_RESTRICT64 : PK_MG_RESTRICT32;
    prof_begin(c, pk, l);
    k_mg_restrict<T><<<g2, b2, 0, c.stream>>>(lview<T>(C, R_<T>(C)), lcview<T>(L, B_<T>(L)), bcf, bcc);
    count_launch(c);
    prof_end(c, pk, l, sizeof(T) * pts * (1.0 + 1.0 / 8.0));
    return chk(c, "mg restrict");
}

template <typename T>
static int prolong_level(Ctx &c, int l, bool tgt, bool add) {
    Level &L = c.lv[l], &C = c.lv[l + 1];
    MgBC bc = level_bc(c, l, tgt);
    dim3 g, b; core_dims(L, g, b);
    int pk = sizeof(T) == 8 ? PK_MG_PROLONG64 : PK_MG_PROLONG32;
    double pts = (double)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1);
    prof_begin(c, pk, l);
    if (tgt && add) {   // the core only: target-mode kernels read face neighbours at their images
        dim3 gm, bm; level_dims<T>(L, gm, bm);
        int sx = (L.n[1] + 3) * (L.n[2] + 3), sy = L.n[2] + 3;
        SARAS_CUDA_TRY(launch_pdl(k_tgt_prolong_add<T>, gm, bm, 0, c.stream, A_<T>(L), A_<T>(C), sx, sy, (C.n[1] + 3) * (C.n[2] + 3),
                                  C.n[2] + 3, bc));
    } else {
        k_mg_prolong_add<T><<<g, b, 0, c.stream>>>(lview<T>(L, A_<T>(L)), lcview<T>(C, A_<T>(C)), bc, add ? 1 : 0);
    }
    count_launch(c);
    prof_end(c, pk, l, sizeof(T) * pts * (2.0 + 1.0 / 8.0));
    return chk(c, "mg prolong");
}

// Sweeps of a smoothing phase below the finest level: coarseSmooth in the
// target modes when set, else the phase's count on the finest level.
static int coarse_sweeps(const Ctx &c, bool tgt, bool pre) {
    if (tgt && c.p.coarseSmooth > 0) return c.p.coarseSmooth;
    return pre ? c.p.preSmooth : c.p.postSmooth;
}

template <typename T>
static int tail_run(Ctx &c, int Lt) {
    TailArgs<T> a;
    a.nl = c.depth - Lt + 1;
    size_t smem = 0;
    for (int q = 0; q < a.nl; ++q) {
        Level &L = c.lv[Lt + q];
        a.bc[q] = level_bc(c, Lt + q, true);
        a.tk[q] = make_tgk<T>(L, 1.0);
        a.tr[q] = make_tgk<T>(L, 1.0);
        smem += 3 * sizeof(T) * (size_t)L.count;
    }
    a.kkc = make_k(c.lv[c.depth]);
    a.M = nullptr;
    a.nM = c.coarseN;
    if (c.coarseN) a.M = sizeof(T) == 8 ? (const T *)c.coarseM64 : (const T *)c.coarseM32;
    a.tol = (T)1.0e-3;   // as coarse_solve in the target modes
    a.maxc = 500;
    int cpre = coarse_sweeps(c, true, true), cpost = coarse_sweeps(c, true, false);
    a.pre = std::min(cpre, kTailMaxSweeps);
    a.post = std::min(cpost, kTailMaxSweeps);
    for (int n = 0; n < kTailMaxSweeps; ++n) {
        a.wpre[n] = (T)smooth_weight(c, n, cpre);
        a.wpost[n] = (T)smooth_weight(c, n, cpost);
    }
    a.rin = R_<T>(c.lv[Lt]);
    a.pout = A_<T>(c.lv[Lt]);
    a.iters = (long long *)(c.dscal + 40);
    SARAS_CUDA_TRY(launch_pdl(k_mg_tail<T>, dim3(1), dim3(kTailThreads), smem, c.stream, a));
    count_launch(c);
    return chk(c, "mg tail");
}

// poisson::vCycle (poisson.cc:219-280) on level arrays of precision T.
// zero0: the level-0 iterate starts at 0 (inner FP32 solve of the mixed mode).
// A cycle from level l down (pre-smoothing, from zero when zero, restriction)
// and back up (prolongation + add, post-smoothing); the levels from the fused
// tail's first one run as that kernel.  gamma cycles on level l + 1 for each
// visit of level l when l == 0 (gamma = 2: a W-cycle at level 1).
template <typename T>
static int cycle_from(Ctx &c, int l, bool tgt, bool zero, int gamma) {
    int s;
    int Lt = tgt ? c.tailLt : -1;   // target modes: levels Lt.. run as one fused kernel
    if (l == Lt) return tail_run<T>(c, Lt);
    if (l == c.depth) return coarse_solve<T>(c, tgt);
    const int pre = l > 0 ? coarse_sweeps(c, tgt, true) : c.p.preSmooth;
    const int post = l > 0 ? coarse_sweeps(c, tgt, false) : c.p.postSmooth;
    if ((s = smooth<T>(c, l, pre, zero, tgt))) return s;
    if ((s = restrict_level<T>(c, l, tgt))) return s;
    const int g = l == 0 ? gamma : 1;
    for (int q = 0; q < g; ++q)
        if ((s = cycle_from<T>(c, l + 1, tgt, q == 0, 1))) return s;
    if ((s = prolong_level<T>(c, l, tgt, true))) return s;
    return smooth<T>(c, l, post, false, tgt);
}

template <typename T>
static int vcycle(Ctx &c, bool tgt, bool zero0) {
    return cycle_from<T>(c, 0, tgt, zero0, tgt ? std::max(1, c.p.coarseCycles) : 1);
}

// The target-mode V-cycle issues about ten kernels per level, most of them
// microseconds long on the coarse levels, where the host's launch rate rather
// than the GPU bounds the cycle.  It is captured once as a CUDA graph and
// replayed: the kernels, their arguments and the level buffers they use are
// the same every cycle, because every level's ping-pong flips an even number
// of times per cycle (pre + post smoothing) and so returns to its starting
// state.  The graph is rebuilt when the level states differ from the ones it
// was captured with; with kernel profiling on, the cycle runs uncaptured.
static std::vector<int> level_state(const Ctx &c, bool timed) {
    std::vector<int> st;
    for (const Level &L : c.lv) { st.push_back(L.cur); st.push_back(L.cur32); }
    for (const ProfSlot &ps : c.prof) st.push_back(timed && ps.enabled ? 1 : 0);   // the profiling event nodes it holds
    return st;
}

static bool any_profiling(const Ctx &c) {
    for (const ProfSlot &ps : c.prof)
        if (ps.enabled) return true;
    return false;
}

static void vgraph_drop(Ctx &c, int a, int b, int t) {
    if (c.vgraph[a][b][t]) cudaGraphExecDestroy(c.vgraph[a][b][t]);
    if (c.vgraphSrc[a][b][t]) cudaGraphDestroy(c.vgraphSrc[a][b][t]);
    for (ProfNode &n : c.vgraphProf[a][b][t]) cudaEventDestroy(n.captured);
    c.vgraph[a][b][t] = nullptr;
    c.vgraphSrc[a][b][t] = nullptr;
    c.vgraphProf[a][b][t].clear();
}

void vgraph_reset(Ctx &c) {
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int t = 0; t < 2; ++t) vgraph_drop(c, a, b, t);
}

// The event-record nodes of graph g that carry the profiling events recorded
// during its capture, in capture order.
static int map_prof_nodes(Ctx &c, cudaGraph_t g, std::vector<ProfNode> &out) {
    out = c.profCaptured;
    c.profCaptured.clear();
    if (out.empty()) return SARAS_OK;
    size_t n = 0;
    SARAS_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    SARAS_CUDA_TRY(cudaGraphGetNodes(g, nodes.data(), &n));
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        SARAS_CUDA_TRY(cudaGraphNodeGetType(nd, &t));
        if (t != cudaGraphNodeTypeEventRecord) continue;
        cudaEvent_t ev;
        SARAS_CUDA_TRY(cudaGraphEventRecordNodeGetEvent(nd, &ev));
        for (ProfNode &p : out)
            if (p.captured == ev) p.node = nd;
    }
    for (const ProfNode &p : out)
        if (!p.node) { c.err = "V-cycle graph: profiling event node not found"; return SARAS_CUDA_ERROR; }
    return SARAS_OK;
}

template <typename T>
static int vcycle_tgt(Ctx &c, bool zero0) {
    // with profiling on, one replay in profEvery runs the instance holding the
    // timing event nodes; the others run an instance captured without them
    const int a = sizeof(T) == 4 ? 1 : 0, b = zero0 ? 1 : 0;
    const int t = any_profiling(c) && (c.profEvery <= 1 || c.profReplays++ % c.profEvery == 0) ? 1 : 0;
    std::vector<int> st = level_state(c, t == 1);
    if (c.vgraph[a][b][t] && c.vgraphState[a][b][t] != st) vgraph_drop(c, a, b, t);
    if (!c.vgraph[a][b][t]) {
        long long l0 = c.launches;
        for (ProfNode &n : c.profCaptured) cudaEventDestroy(n.captured);
        c.profCaptured.clear();
        SARAS_CUDA_TRY(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        c.profCapturing = true;
        c.profSuppress = t == 0;
        int s = vcycle<T>(c, true, zero0);
        c.profCapturing = false;
        c.profSuppress = false;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(c.stream, &g);
        if (s || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            for (ProfNode &n : c.profCaptured) cudaEventDestroy(n.captured);
            c.profCaptured.clear();
            cudaGetLastError();
            if (s) return s;
            c.err = std::string("V-cycle capture: ") + cudaGetErrorString(e);
            return SARAS_CUDA_ERROR;
        }
        c.vgraphSrc[a][b][t] = g;
        if ((s = map_prof_nodes(c, g, c.vgraphProf[a][b][t]))) { vgraph_drop(c, a, b, t); return s; }
        e = cudaGraphInstantiate(&c.vgraph[a][b][t], g, 0);
        if (e != cudaSuccess) {
            c.vgraph[a][b][t] = nullptr;
            vgraph_drop(c, a, b, t);
            c.err = std::string("V-cycle graph: ") + cudaGetErrorString(e);
            return SARAS_CUDA_ERROR;
        }
        c.vgraphLaunches[a][b][t] = c.launches - l0;
        c.launches = l0;
        c.vgraphState[a][b][t] = st;
        if (level_state(c, t == 1) != st) {   // a cycle that does not restore the level states is never replayed:
            vgraph_drop(c, a, b, t);          // back to the states before the capture, then run it directly
            for (size_t q = 0; q < c.lv.size(); ++q) { c.lv[q].cur = st[2 * q]; c.lv[q].cur32 = st[2 * q + 1]; }
            return vcycle<T>(c, true, zero0);
        }
    }
    int s = prof_graph_replay(c, c.vgraph[a][b][t], c.vgraphProf[a][b][t]);
    if (s) { c.err = "V-cycle graph: profiling events"; return s; }
    SARAS_CUDA_TRY(cudaGraphLaunch(c.vgraph[a][b][t], c.stream));
    c.launches += c.vgraphLaunches[a][b][t];
    return SARAS_OK;
}

static int read_scalars(Ctx &c, int first, int count) {
    SARAS_CUDA_TRY(cudaMemcpyAsync(c.hscal + first, c.dscal + first, sizeof(double) * count, cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return SARAS_OK;
}

static int grid_blocks(long n) { return (int)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 8)); }

int mg_compute_error(Ctx &c, int norm, double *err) {
    Level &L = c.lv[0];
    MgBC bc = level_bc(c, 0, false);
    MgK kk = make_k(L);
    long n = (long)(L.n[0] + 1) * (L.n[1] + 1) * (L.n[2] + 1);
    int nb = std::min(grid_blocks(n), c.redCap);
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 22, 0, sizeof(double), c.stream));
    // denominator max|residualData(0)| over the padded array (poisson_d3.cc:437)
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 21, 0, sizeof(double), c.stream));
    if (norm == 1) {
        k_maxabs<<<grid_blocks(L.count), 256, 0, c.stream>>>(L.r, L.count, c.dscal + 21);
        count_launch(c);
    }
    if (norm == 1) {
        k_mg_error<<<nb, 256, 0, c.stream>>>(lcview<double>(L, L.pa()), lcview<double>(L, L.r), kk, bc, norm, c.dscal + 22, c.red,
                                             c.red + c.redCap);
        count_launch(c);
    } else {
        long nch = (n + kChunk - 1) / kChunk;
        if (nch > c.redCap) { c.err = "reduction buffer too small"; return SARAS_TOO_LARGE; }
        k_mg_error_sq<<<(int)((nch + 127) / 128), 128, 0, c.stream>>>(lcview<double>(L, L.pa()), lcview<double>(L, L.r), kk, bc,
                                                                      c.red, c.red + c.redCap);
        k_seq_sum<<<1, 32, 0, c.stream>>>(c.red, nch, c.dscal + 24);
        k_seq_sum<<<1, 32, 0, c.stream>>>(c.red + c.redCap, nch, c.dscal + 25);
        count_launch(c, 3);
    }
    int s = chk(c, "computeError");
    if (s) return s;
    if ((s = read_scalars(c, 21, 5))) return s;
    double e = 0;
    if (norm == 1) {
        double num = c.hscal[22], den = c.hscal[21];
        e = den ? num / den : num;
    } else if (norm == 2) {
        double cnt = (double)n;
        double num = c.hscal[24], den = c.hscal[25];
        e = den ? std::sqrt(num / cnt) / std::sqrt(den / cnt) : std::sqrt(num / cnt);
    }
    *err = e;
    return SARAS_OK;
}

// poisson::mgSolve (poisson.cc:100-205), reference mode.
static int mg_solve_reference(Ctx &c, int *cycles, double *residual) {
    int s;
    Level &L0 = c.lv[0];
    MgBC bc0 = level_bc(c, 0, false);
    // zero scalars used for the |r| denominator and the mean offset trick
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 20, 0, sizeof(double) * 8, c.stream));
    int nb = std::min(grid_blocks(L0.count), c.redCap);
    View3<const double> rhs = lcview<double>(L0, c.f[SARAS_FIELD_MGRHS]);
    k_mg_load<<<nb, 256, 0, c.stream>>>(lview<double>(L0, L0.r), rhs, bc0, c.red);
    count_launch(c);
    if (!c.p.testPoisson) {
        long nch = (L0.count + kChunk - 1) / kChunk;
        if (nch > c.redCap) { c.err = "reduction buffer too small"; return SARAS_TOO_LARGE; }
        k_chunk_sum_flat<<<(int)((nch + 127) / 128), 128, 0, c.stream>>>(L0.r, L0.count, c.red);
        k_seq_sum<<<1, 32, 0, c.stream>>>(c.red, nch, c.dscal + 20);
        k_mg_sub_mean<<<grid_blocks(L0.count), 256, 0, c.stream>>>(L0.r, L0.count, c.dscal + 20, (double)L0.count, c.dscal + 27);
        count_launch(c, 3);
    }
    // pressureData(0)(core) = Pp(core) (+ face ghosts)
    L0.cur = 0;
    dim3 g, b; core_dims(L0, g, b);
    k_mg_init_p<double><<<g, b, 0, c.stream>>>(lview<double>(L0, L0.pa()), lcview<double>(L0, c.f[SARAS_FIELD_PP]), bc0);
    count_launch(c);
    if (c.p.testPoisson) {
        dim3 g2, b2;
        Level tmp = L0; tmp.n[0] += 2; tmp.n[1] += 2; tmp.n[2] += 2;
        core_dims(tmp, g2, b2);
        k_dirichlet_walls<<<g2, b2, 0, c.stream>>>(lview<double>(L0, L0.a), bc0, c.wallX, c.wallY, c.wallZ);
        k_dirichlet_walls<<<g2, b2, 0, c.stream>>>(lview<double>(L0, L0.b), bc0, c.wallX, c.wallY, c.wallZ);
        count_launch(c, 2);
    }
    if ((s = chk(c, "mg load"))) return s;
    double prev = 0.0, res = 0.0;
    int cyc = 0;
    for (int i = 0; i < c.p.vcCount; ++i) {
        if ((s = vcycle<double>(c, false, false))) return s;
        cyc += 1;
        if ((s = mg_compute_error(c, c.p.resType, &res))) return s;
        if (!std::isfinite(res)) { c.err = "multigrid residual is not finite"; return SARAS_NOT_FINITE; }
        if (!c.p.testPoisson) {
            if (std::fabs(prev - res) < c.p.mgTolerance) break;
            prev = res;
        }
    }
    if (c.p.gsSmooth && (s = gs_status(c))) return s;
    // inFn.F = pressureData(0) over the padded array (poisson.cc:151)
    k_mg_output<<<grid_blocks(L0.count), 256, 0, c.stream>>>(lview<double>(L0, c.f[SARAS_FIELD_PP]), lcview<double>(L0, L0.pa()), bc0,
                                                             c.wallX, c.wallY, c.wallZ);
    count_launch(c);
    if ((s = chk(c, "mg output"))) return s;
    if (cycles) *cycles = cyc;
    if (residual) *residual = res;
    return SARAS_OK;
}

// SARAS_MG_MIXED on an isotropic level 0: FP32 V-cycles inside the exact
// fixed-point refinement (k_fx_refine).  On entry L0.r holds b, L0.pa() the
// previous Pp with its face ghosts.  On return with done = true, L0.pa() holds
// the FP64 result, r its residual max|b - A p| (evaluated exactly on the FP64
// values), and the counters are set.  done = false (a value left the
// fixed-point range, which takes a diverging iterate) leaves L0.pa() holding
// the previous Pp again for the FP64 refinement loop.
constexpr int kMaxAdaptiveCycles = 8;   // V-cycles in one refinement step at most (mixedCycles = 0)

// V-cycles of the next refinement step from residual r.  The first step of a
// solve runs mixedCycles cycles; a later step (the target was missed), or any
// step with mixedCycles = 0, runs the fewest that the measured contraction per
// cycle predicts to reach the target, at most mixedCycles (kMaxAdaptiveCycles
// for 0); never beyond mgMaxCycles in total.
static int refine_cycles(const Ctx &c, double r, double target, int cyc, bool first) {
    int cap = c.p.mixedCycles > 0 ? c.p.mixedCycles : kMaxAdaptiveCycles;
    int n = cap;
    if (!(first && c.p.mixedCycles > 0)) {
        double need = std::log(target / r) / std::log(c.rhoMixed);
        n = std::isfinite(need) ? std::max(1, std::min(cap, (int)std::ceil(need - 1e-3))) : 1;
    }
    return std::min(n, std::max(1, c.mgMaxCycles - cyc));
}

// Running estimate of the contraction per FP32 V-cycle from one refinement
// step (r0 -> r over n cycles), kept within [0.005, 0.5].
static void note_contraction(Ctx &c, double r0, double r, int n) {
    if (!(r0 > 0.0) || !(r > 0.0) || !std::isfinite(r) || !std::isfinite(r0)) return;
    double rho = std::pow(r / r0, 1.0 / n);
    c.rhoMixed = std::min(0.5, std::max(0.005, 0.5 * c.rhoMixed + 0.5 * rho));
}

// A guess whose residual is at most this fraction of max|b| starts the solve
// without a comparison against the previous Pp (whose residual is the whole
// change of b over the step).  Extrapolated guesses measured a few 1e-6 of
// max|b| on the 257^3 Taylor-Green vortex; below 1e-4 the two starts differ
// by a cycle at most.
constexpr double kGuessTrusted = 1e-4;

static int mixed_fixed(Ctx &c, const double *pp0, double mean, double bmax, double pmax, double target, bool wantGuess, double &r, int &source,
                       int &cyc, int &steps, bool &done, saras_step_stats *st) {
    int s;
    Level &L0 = c.lv[0];
    MgBC bc0 = level_bc(c, 0, true);
    done = false;
    for (long long *&q : c.fx)
        if (!q) {
            SARAS_CUDA_TRY(cudaMalloc(&q, sizeof(long long) * L0.count));
            SARAS_CUDA_TRY(cudaMemsetAsync(q, 0, sizeof(long long) * L0.count, c.stream));
        }
    long long *B = c.fx[2];
    unsigned long long *dmax = reinterpret_cast<unsigned long long *>(c.dscal + 34);
    int *dflag = reinterpret_cast<int *>(c.dscal + 35);
    // scale: |P|, |B| <= 2^55 for the largest of max|p| (the padded Pp) and max|b| / l
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 34, 0, sizeof(double) * 2, c.stream));
    double l = L0.lx;
    double M = std::max(pmax, bmax / l);
    int sx0 = (L0.n[1] + 3) * (L0.n[2] + 3), sy0 = L0.n[2] + 3;
    dim3 gk0, bk0; col_dims(L0, gk0, bk0);
    const double *rhs = c.f[SARAS_FIELD_MGRHS];
    // the FP64 path's start (b in level-0 r, p = Pp) when the fixed-point path gives up
    bool bDone = false;
    auto fp64_start = [&]() -> int {
        dim3 gi, bi; core_dims(L0, gi, bi);
        if (!bDone) k_tgt_rhs<<<gk0, bk0, 0, c.stream>>>(L0.r, rhs, sx0, sy0, bc0, mean);
        k_mg_init_p<double><<<gi, bi, 0, c.stream>>>(lview<double>(L0, L0.pa()), lcview<double>(L0, pp0), bc0);
        count_launch(c, bDone ? 1 : 2);
        return chk(c, "fixed-point fallback");
    };
    if (!(M > 0.0) || !std::isfinite(M)) return fp64_start();   // nothing to scale (or not finite)
    int sc = 54 - std::ilogb(M);
    sc = std::max(-900, std::min(900, sc));
    double inv2s = std::ldexp(1.0, -sc);
    double rs = l * inv2s;   // residual units -> value
    dim3 gm0, bm0; march_dims(L0, gm0, bm0);
    dim3 gc, bcd; core_dims(L0, gc, bcd);
    // b itself only where it is read: the learned guess's restricted history, and pairs collected for training
    bDone = c.collecting || unet_tracking(c);
    k_fx_rhs<<<gk0, bk0, 0, c.stream>>>(B, bDone ? L0.r : nullptr, rhs, sx0, sy0, bc0, mean, std::ldexp(1.0, sc) / l, dflag);
    count_launch(c);
    // With Pp's buffer free for the output (the previous Pp is pHist[0]), every
    // refinement update writes its FP64 iterate into Pp's core as it goes.
    double *outp = c.ppInHist ? c.f[SARAS_FIELD_PP] : nullptr;
    // residual of fixed iterate q (with e: advanced into q ^ 1 first); returns the max in value units
    auto refine = [&](int q, bool withE, double &out, bool &bad, bool fill32 = true) -> int {
        SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 34, 0, sizeof(double), c.stream));
        if (withE) {
            prof_begin(c, PK_REFINE_UPDATE, 0);
            k_fx_update<<<gm0, bm0, 0, c.stream>>>(c.fx[q ^ 1], c.fx[q], L0.pa32(), B, L0.r32, sx0, sy0, bc0, sc, (float)rs, dmax, dflag,
                                                   outp, inv2s);
            prof_end(c, PK_REFINE_UPDATE, 0, (8.0 + 4.0 + 8.0 + 8.0 + 4.0 + (outp ? 8.0 : 0.0)) * (double)L0.count);
        } else {
            prof_begin(c, PK_REFINE_RESID, 0);
            k_fx_refine<<<gk0, bk0, 0, c.stream>>>(c.fx[q], B, fill32 ? L0.r32 : nullptr, sx0, sy0, bc0, (float)rs, dmax);
            prof_end(c, PK_REFINE_RESID, 0, (8.0 + 8.0 + (fill32 ? 4.0 : 0.0)) * (double)L0.count);
        }
        count_launch(c);
        int e = chk(c, "fixed-point refinement");
        if (e) return e;
        unsigned long long mx = 0;
        int fl = 0, tmaErr = 0;
        SARAS_CUDA_TRY(cudaMemcpyAsync(&mx, dmax, sizeof(mx), cudaMemcpyDeviceToHost, c.stream));
        SARAS_CUDA_TRY(cudaMemcpyAsync(&fl, dflag, sizeof(fl), cudaMemcpyDeviceToHost, c.stream));
        if (c.planeOk) SARAS_CUDA_TRY(cudaMemcpyAsync(&tmaErr, c.dflag + 2, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
        if (tmaErr) { c.err = "plane-streaming stencil: an mbarrier wait timed out"; return SARAS_CUDA_ERROR; }
        out = (double)mx * rs;
        bad = fl != 0;
        return SARAS_OK;
    };
    bool bad = false;
    int built = 0;
    int cur = 0;
    // the start: a guess whose residual is at most kGuessTrusted max|b| is
    // taken as it is; otherwise (or with no guess) the previous Pp's residual
    // is computed too and the smaller one starts the solve
    bool started = false;
    double rg = 0;
    int gs = SARAS_BAD_CONFIG, gq = 1;   // gq: the fixed-point iterate holding the guess
    if (wantGuess && c.histCount >= 2) {
        built = unet_pick(c);
        prof_begin(c, PK_GUESS, 0);
        gs = unet_guess(c, L0.r, nullptr, built, c.fx[1], sc, dflag);
        prof_end(c, PK_GUESS, 0, 0.0);
        if (gs == SARAS_OK) {
            if ((s = refine(1, false, rg, bad))) return s;
            if (bad) return fp64_start();
            unet_note_start(c, built, rg / bmax);
            // the learned mode's probes build the other guess too; the better starts
            if (const int other = unet_shadow(c, built)) {
                prof_begin(c, PK_GUESS, 0);
                const int go = unet_guess(c, L0.r, nullptr, other, c.fx[0], sc, dflag);
                prof_end(c, PK_GUESS, 0, 0.0);
                if (go == SARAS_OK) {
                    double ro = 0;
                    if ((s = refine(0, false, ro, bad, false))) return s;   // its max only; r32 keeps the first guess's
                    if (bad) return fp64_start();
                    unet_note_start(c, other, ro / bmax);
                    if (ro < rg) {
                        if ((s = refine(0, false, ro, bad))) return s;      // its FP32 residual into r32
                        if (bad) return fp64_start();
                        rg = ro;
                        built = other;
                        gq = 0;
                    }
                } else if (go != SARAS_BAD_CONFIG) {
                    return go;
                }
            }
            if (rg <= kGuessTrusted * bmax) {
                r = rg;
                source = built;
                cur = gq;
                started = true;
            }
        } else if (gs != SARAS_BAD_CONFIG) {
            return gs;
        }
    }
    if (!started) {
        const int pq = gq ^ 1;   // the previous Pp into the other iterate
        k_fx_init<<<gc, bcd, 0, c.stream>>>(c.fx[pq], lcview<double>(L0, pp0), bc0, sc, dflag);
        count_launch(c);
        if ((s = refine(pq, false, r, bad))) return s;
        if (bad) return fp64_start();
        cur = pq;
        if (gs == SARAS_OK && rg < r) {   // the guess after all: its FP32 residual back into r32
            if ((s = refine(gq, false, rg, bad))) return s;
            if (bad) return fp64_start();
            r = rg;
            source = built;
            cur = gq;
        }
    }
    if (st) { st->guess_residual = bmax > 0 ? r / bmax : r; st->guess_source = source; }
    bool updated = false;
    while (r > target && cyc < c.mgMaxCycles) {
        if (!std::isfinite(r)) { c.err = "multigrid residual is not finite"; return SARAS_NOT_FINITE; }
        int n = refine_cycles(c, r, target, cyc, steps == 0);
        double r0 = r;
        for (int q = 0; q < n; ++q) {
            if ((s = vcycle_tgt<float>(c, q == 0))) return s;
            cyc += 1;
        }
        steps += 1;
        if ((s = refine(cur, true, r, bad))) return s;
        if (bad) break;
        cur ^= 1;
        updated = true;
        note_contraction(c, r0, r, n);
    }
    if (!bad) {
        // the FP64 result P 2^-s (exact), whose exact residual is r
        if (updated && outp) {   // the core is written: the ghost positions
            int most = 0;   // padded points of the largest face
            for (int d = 0; d < 3; ++d) most = std::max(most, (L0.n[(d + 1) % 3] + 3) * (L0.n[(d + 2) % 3] + 3));
            k_fx_output_shell<<<dim3((most + 255) / 256, 1, 6), 256, 0, c.stream>>>(outp, c.fx[cur], bc0, inv2s);
        } else {
            dim3 bo(64, 4, 1), go((L0.n[2] + 3 + 63) / 64, (L0.n[1] + 3 + 3) / 4, L0.n[0] + 3);
            k_fx_output<<<go, bo, 0, c.stream>>>(c.f[SARAS_FIELD_PP], c.fx[cur], bc0, inv2s);
        }
        count_launch(c);
        c.ppInHist = false;
        done = true;
        return chk(c, "fixed-point output");
    }
    // out of range: restart from the previous Pp in FP64
    L0.cur = 0;
    r = 0; source = 0; cyc = 0; steps = 0;
    return fp64_start();
}

// Target modes: plain FP64 V-cycles or FP32 V-cycles inside FP64 refinement.
static int mg_solve_target_run(Ctx &c, int *cycles, double *residual, saras_step_stats *st) {
    int s;
    Level &L0 = c.lv[0];
    MgBC bc0 = level_bc(c, 0, true);
    dim3 g, b; core_dims(L0, g, b);
    long ncore = (long)(L0.n[0] + 1) * (L0.n[1] + 1) * (L0.n[2] + 1);
    int nb = std::min(grid_blocks(ncore), c.redCap);
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 30, 0, sizeof(double) * 6, c.stream));
    // pressure history for the learned / extrapolated guess
    bool wantGuess = c.guessMode != SARAS_GUESS_PREVIOUS;
    if (wantGuess || c.collecting) {
        prof_begin(c, PK_GUESS, 0);
        s = unet_begin_solve(c);
        prof_end(c, PK_GUESS, 0, 0.0);
        if (s) return s;
    }
    const double *pp0 = c.ppInHist ? c.pHist[0] : c.f[SARAS_FIELD_PP];   // the previous Pp
    const double *rhs = c.f[SARAS_FIELD_MGRHS];
    // the fixed-point path forms b = rhs - trapezoidal mean itself and needs
    // max|Pp| for its scale; the FP64 path stores b in level-0 r and starts
    // from p = Pp with face ghosts
    bool fixedPath = c.mgMode == SARAS_MG_MIXED && L0.lx == L0.ly && L0.ly == L0.lz;
    int sx0 = (L0.n[1] + 3) * (L0.n[2] + 3), sy0 = L0.n[2] + 3;
    dim3 gk0, bk0; col_dims(L0, gk0, bk0);
    int nparts = (int)(gk0.x * gk0.y);
    if (nparts > c.redCap) { c.err = "reduction buffer too small"; return SARAS_TOO_LARGE; }
    k_tgt_stats<<<gk0, bk0, 0, c.stream>>>(lcview<double>(L0, rhs), fixedPath ? pp0 : nullptr, bc0, c.red, c.dscal + 31, c.dscal + 32,
                                           c.dscal + 33);
    k_final_reduce<<<1, 256, 0, c.stream>>>(c.red, nparts, 0, c.dscal + 30);
    count_launch(c, 2);
    if ((s = chk(c, "target load"))) return s;
    if ((s = read_scalars(c, 30, 4))) return s;
    double wsum = 1.0;
    for (int d = 0; d < 3; ++d) wsum *= (double)L0.n[d];
    const double mean = c.hscal[30] * (1.0 / wsum);
    double bmax, pmax = c.hscal[33];
    {
        unsigned long long kh, kl;
        std::memcpy(&kh, &c.hscal[31], sizeof kh);
        std::memcpy(&kl, &c.hscal[32], sizeof kl);
        const double up = order_key_value(kh) - mean, dn = mean - order_key_value(~kl);
        bmax = (std::isnan(up) || std::isnan(dn)) ? up + dn : std::max(up, dn);
    }
    L0.cur = 0;
    if (!fixedPath) {
        dim3 g, b; core_dims(L0, g, b);
        k_tgt_rhs<<<gk0, bk0, 0, c.stream>>>(L0.r, rhs, sx0, sy0, bc0, mean);
        k_mg_init_p<double><<<g, b, 0, c.stream>>>(lview<double>(L0, L0.pa()), lcview<double>(L0, pp0), bc0);
        count_launch(c, 2);
    }
    double target = c.mgTarget * bmax;
    TgK<double> t0 = make_tgk<double>(L0, 1.0);
    dim3 gm0, bm0; march_dims(L0, gm0, bm0);
    auto fine_res = [&](bool withE, double *out) -> int {
        SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 32, 0, sizeof(double), c.stream));
        if (withE) {
            prof_begin(c, PK_REFINE_UPDATE, 0);
            k_tgt_update<<<gm0, bm0, 0, c.stream>>>(L0.pa(), L0.pa32(), sx0, sy0, bc0);
            count_launch(c);
            prof_end(c, PK_REFINE_UPDATE, 0, (8.0 + 4.0 + 8.0) * (double)ncore);
        }
        prof_begin(c, PK_REFINE_RESID, 0);
        if (c.mgMode == SARAS_MG_MIXED) {
            k_tgt_residual<double, float, true><<<gk0, bk0, 0, c.stream>>>(L0.r32, L0.pa(), L0.r, sx0, sy0, bc0, t0, c.dscal + 32);
            prof_end(c, PK_REFINE_RESID, 0, (8.0 + 8.0 + 4.0) * (double)ncore);
        } else {
            k_tgt_residual<double, double, true><<<gk0, bk0, 0, c.stream>>>(nullptr, L0.pa(), L0.r, sx0, sy0, bc0, t0, c.dscal + 32);
            prof_end(c, PK_REFINE_RESID, 0, (8.0 + 8.0) * (double)ncore);
        }
        count_launch(c);
        int q = chk(c, "refine");
        if (q) return q;
        q = read_scalars(c, 32, 1);
        if (q) return q;
        *out = c.hscal[32];
        return SARAS_OK;
    };
    double r = 0;
    int source = 0, cyc = 0, steps = 0, built = 0;
    bool fixedDone = false;
    if (fixedPath) {
        if ((s = mixed_fixed(c, pp0, mean, bmax, pmax, target, wantGuess, r, source, cyc, steps, fixedDone, st))) return s;
    }
    if (!fixedDone) {
    if ((s = fine_res(false, &r))) return s;
    if (wantGuess && c.histCount >= 2) {
        built = unet_pick(c);
        unet_shadow(c, built);   // one guess at a time on this path
        int gs = unet_guess(c, L0.r, L0.pb(), built);
        if (gs == SARAS_OK) {
            L0.cur ^= 1;
            double rg = 0;
            if ((s = fine_res(false, &rg))) return s;
            unet_note_start(c, built, rg / bmax);
            if (rg < r) {
                r = rg;
                source = built;
            } else {
                L0.cur ^= 1;   // keep the previous pressure (and recompute its FP32 residual)
                if ((s = fine_res(false, &r))) return s;
            }
        } else if (gs != SARAS_BAD_CONFIG) {
            return gs;
        }
    }
    if (st) { st->guess_residual = bmax > 0 ? r / bmax : r; st->guess_source = source; }
    while (r > target && cyc < c.mgMaxCycles) {
        if (!std::isfinite(r)) { c.err = "multigrid residual is not finite"; return SARAS_NOT_FINITE; }
        if (c.mgMode == SARAS_MG_PLAIN_TARGET) {
            if ((s = vcycle_tgt<double>(c, false))) return s;
            cyc += 1;
            if ((s = fine_res(false, &r))) return s;
        } else {
            // inner FP32 solve of A e = r32 from e = 0
            int n = refine_cycles(c, r, target, cyc, steps == 0);
            double r0 = r;
            for (int q = 0; q < n; ++q) {
                if ((s = vcycle_tgt<float>(c, q == 0))) return s;
                cyc += 1;
            }
            steps += 1;
            if ((s = fine_res(true, &r))) return s;
            note_contraction(c, r0, r, n);
        }
    }
    }
    if (st) { st->refine_steps = steps; st->fine_residual = bmax > 0 ? r / bmax : r; }
    if (!fixedDone) {   // the fixed-point path has written Pp already (k_fx_output)
        k_mg_output<<<grid_blocks(L0.count), 256, 0, c.stream>>>(lview<double>(L0, c.f[SARAS_FIELD_PP]), lcview<double>(L0, L0.pa()), bc0,
                                                                 nullptr, nullptr, nullptr);
        count_launch(c);
        c.ppInHist = false;
    }
    if ((s = chk(c, "target output"))) return s;
    if (c.collecting && r <= target) {
        if ((s = unet_collect_sample(c, L0.r))) return s;
    }
    if (cycles) *cycles = cyc;
    if (residual) *residual = bmax > 0 ? r / bmax : r;
    if (r > target) { c.err = "multigrid did not reach the residual target within mgMaxCycles"; return SARAS_NOT_CONVERGED; }
    return SARAS_OK;
}

// A solve that ends before writing Pp leaves the previous Pp in place.
static int mg_solve_target(Ctx &c, int *cycles, double *residual, saras_step_stats *st) {
    int s = mg_solve_target_run(c, cycles, residual, st);
    if (c.ppInHist) {
        c.ppInHist = false;
        SARAS_CUDA_TRY(cudaMemcpyAsync(c.f[SARAS_FIELD_PP], c.pHist[0], sizeof(double) * c.lv[0].count, cudaMemcpyDeviceToDevice, c.stream));
    }
    return s;
}

int mg_solve(Ctx &c, int *cycles, double *residual, saras_step_stats *st) {
    long long before = 0;
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 40, 0, sizeof(double), c.stream));
    int s = c.mgMode == SARAS_MG_REFERENCE ? mg_solve_reference(c, cycles, residual) : mg_solve_target(c, cycles, residual, st);
    if (s) return s;
    if (c.mgMode != SARAS_MG_REFERENCE && c.tailLt >= 0 && c.coarseN > 0) {
        // the coarsest level is solved by its operator: no Gauss-Seidel
        // iterations to count, and no synchronisation to read them
        if (st) st->coarse_iters = 0;
        return SARAS_OK;
    }
    SARAS_CUDA_TRY(cudaMemcpyAsync(&before, c.dscal + 40, sizeof(long long), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    c.coarseIters += before;
    if (st) st->coarse_iters = (int)before;
    return SARAS_OK;
}

// ---- test hooks mirroring the protected multigrid_d3 methods
int mg_set_level(Ctx &c, int level, int which, const double *host) {
    if (level < 0 || level > c.depth || (which != 0 && which != 1)) return SARAS_BAD_ARG;
    Level &L = c.lv[level];
    double *dst = which == 0 ? L.pa() : L.r;
    SARAS_CUDA_TRY(cudaMemcpyAsync(dst, host, sizeof(double) * L.count, cudaMemcpyHostToDevice, c.stream));
    if (which == 0) {
        // keep the face ghosts consistent with imposeBC, as smooth() would on entry
        MgBC bc = level_bc(c, level, false);
        dim3 g, b; core_dims(L, g, b);
        k_mg_init_p<double><<<g, b, 0, c.stream>>>(lview<double>(L, L.pb()), lcview<double>(L, dst), bc);
        count_launch(c);
        L.cur ^= 1;
    }
    return chk(c, "set level");
}

int mg_get_level(Ctx &c, int level, int which, double *host) {
    if (level < 0 || level > c.depth || (which != 0 && which != 1)) return SARAS_BAD_ARG;
    Level &L = c.lv[level];
    const double *src = which == 0 ? L.pa() : L.r;
    SARAS_CUDA_TRY(cudaMemcpyAsync(host, src, sizeof(double) * L.count, cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return SARAS_OK;
}

int mg_smooth_level(Ctx &c, int level, int count) {
    if (level < 0 || level > c.depth) return SARAS_BAD_ARG;
    if (level == c.depth && count < 0) return coarse_solve<double>(c, false);
    int s = smooth<double>(c, level, count, false, false);
    if (!s && c.p.gsSmooth) s = gs_status(c);
    return s;
}

int mg_restrict_level(Ctx &c, int level) {
    if (level < 0 || level >= c.depth) return SARAS_BAD_ARG;
    return restrict_level<double>(c, level, false);
}

int mg_prolong_level(Ctx &c, int level) {
    if (level < 0 || level >= c.depth) return SARAS_BAD_ARG;
    return prolong_level<double>(c, level, false, true);
}

// multigrid_d3::testProlong (poisson_d3.cc:689-719)
int mg_test_prolong(Ctx &c, double *err) {
    if (c.depth < 1) return SARAS_BAD_ARG;
    Level &L0 = c.lv[0], &L1 = c.lv[1];
    std::vector<double> h1(L1.count, 0.0), h0(L0.count, 0.0);
    View3<double> v1 = lview<double>(L1, nullptr), v0 = lview<double>(L0, nullptr);
    // linear function sampled at the coincident fine indices (2i, 2j, 2k)
    for (int i = 0; i <= L1.n[0]; ++i) for (int j = 0; j <= L1.n[1]; ++j) for (int k = 0; k <= L1.n[2]; ++k)
        h1[v1.off(i, j, k)] = 1000 + (2 * i) * 100 + (2 * j) * 10 + 2 * k;
    for (int i = 0; i <= L0.n[0]; ++i) for (int j = 0; j <= L0.n[1]; ++j) for (int k = 0; k <= L0.n[2]; ++k)
        h0[v0.off(i, j, k)] = 1000 + i * 100 + j * 10 + k;
    SARAS_CUDA_TRY(cudaMemcpyAsync(L1.pa(), h1.data(), L1.count * 8, cudaMemcpyHostToDevice, c.stream));
    SARAS_CUDA_TRY(cudaMemsetAsync(L0.pa(), 0, L0.count * 8, c.stream));
    MgBC bc = level_bc(c, 0, false);
    dim3 g, b; core_dims(L0, g, b);
    k_mg_prolong_add<double><<<g, b, 0, c.stream>>>(lview<double>(L0, L0.pa()), lcview<double>(L1, L1.pa()), bc, 0);
    count_launch(c);
    std::vector<double> out(L0.count);
    SARAS_CUDA_TRY(cudaMemcpyAsync(out.data(), L0.pa(), L0.count * 8, cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    double m = 0;
    for (int i = 0; i <= L0.n[0]; ++i) for (int j = 0; j <= L0.n[1]; ++j) for (int k = 0; k <= L0.n[2]; ++k)
        m = std::max(m, std::fabs(out[v0.off(i, j, k)] - h0[v0.off(i, j, k)]));
    *err = m;
    return SARAS_OK;
}

// multigrid_d3::testTransfer (poisson_d3.cc:722-777) at level 0: face pads
// after updatePads, for periodic x and y.
int mg_test_transfer(Ctx &c, double *err) {
    Level &L0 = c.lv[0];
    View3<double> v0 = lview<double>(L0, nullptr);
    std::vector<double> h(L0.count, 0.0), e(L0.count, 0.0);
    int X = L0.n[0], Y = L0.n[1], Z = L0.n[2];
    for (int i = 0; i <= X; ++i) for (int j = 0; j <= Y; ++j) for (int k = 0; k <= Z; ++k)
        h[v0.off(i, j, k)] = e[v0.off(i, j, k)] = 1000 + i * 100 + j * 10 + k;
    for (int j = 0; j <= Y; ++j) for (int k = 0; k <= Z; ++k) {
        e[v0.off(-1, j, k)] = 1000 + (X - 1) * 100 + j * 10 + k;
        e[v0.off(X + 1, j, k)] = 1000 + 100 + j * 10 + k;
    }
    for (int i = 0; i <= X; ++i) for (int k = 0; k <= Z; ++k) {
        e[v0.off(i, -1, k)] = 1000 + i * 100 + (Y - 1) * 10 + k;
        e[v0.off(i, Y + 1, k)] = 1000 + i * 100 + 10 + k;
    }
    SARAS_CUDA_TRY(cudaMemcpyAsync(L0.pb(), h.data(), L0.count * 8, cudaMemcpyHostToDevice, c.stream));
    MgBC bc = level_bc(c, 0, false);
    dim3 g, b; core_dims(L0, g, b);
    k_mg_init_p<double><<<g, b, 0, c.stream>>>(lview<double>(L0, L0.pa()), lcview<double>(L0, L0.pb()), bc);
    count_launch(c);
    std::vector<double> out(L0.count);
    SARAS_CUDA_TRY(cudaMemcpyAsync(out.data(), L0.pa(), L0.count * 8, cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    double m = 0;
    for (int i = -1; i <= X + 1; ++i) for (int j = -1; j <= Y + 1; ++j) for (int k = 0; k <= Z; ++k) {
        int gi = (i < 0 || i > X), gj = (j < 0 || j > Y);
        if (gi && gj) continue;
        m = std::max(m, std::fabs(out[v0.off(i, j, k)] - e[v0.off(i, j, k)]));
    }
    *err = m;
    return SARAS_OK;
}

// multigrid_d3::testPeriodic (poisson_d3.cc:780-857) at level 0: face ghosts
// of sin*cos*cos after imposeBC.
int mg_test_periodic(Ctx &c, double *err) {
    Level &L0 = c.lv[0];
    View3<double> v0 = lview<double>(L0, nullptr);
    int X = L0.n[0], Y = L0.n[1], Z = L0.n[2];
    std::vector<double> h(L0.count, 0.0), e(L0.count, 0.0);
    const double PI = M_PI;
    auto xs = [&](int d, int i) { return c.L[d] * (double(i) * c.dXi[d]); };
    auto fn = [&](double x, double y, double z) {
        return std::sin(2.0 * PI * x / c.L[0]) * std::cos(2.0 * PI * y / c.L[1]) * std::cos(2.0 * PI * z / c.L[2]);
    };
    for (int i = 0; i <= X; ++i) for (int j = 0; j <= Y; ++j) for (int k = 0; k <= Z; ++k)
        h[v0.off(i, j, k)] = e[v0.off(i, j, k)] = fn(xs(0, i), xs(1, j), xs(2, k));
    for (int j = 0; j <= Y; ++j) for (int k = 0; k <= Z; ++k) {
        e[v0.off(-1, j, k)] = fn(xs(0, 0) - (xs(0, 1) - xs(0, 0)), xs(1, j), xs(2, k));
        e[v0.off(X + 1, j, k)] = fn(xs(0, X) + (xs(0, X) - xs(0, X - 1)), xs(1, j), xs(2, k));
    }
    for (int i = 0; i <= X; ++i) for (int k = 0; k <= Z; ++k) {
        e[v0.off(i, -1, k)] = fn(xs(0, i), xs(1, 0) - (xs(1, 1) - xs(1, 0)), xs(2, k));
        e[v0.off(i, Y + 1, k)] = fn(xs(0, i), xs(1, Y) + (xs(1, Y) - xs(1, Y - 1)), xs(2, k));
    }
    for (int i = 0; i <= X; ++i) for (int j = 0; j <= Y; ++j) {
        e[v0.off(i, j, -1)] = fn(xs(0, i), xs(1, j), xs(2, 0) - (xs(2, 1) - xs(2, 0)));
        e[v0.off(i, j, Z + 1)] = fn(xs(0, i), xs(1, j), xs(2, Z) + (xs(2, Z) - xs(2, Z - 1)));
    }
    SARAS_CUDA_TRY(cudaMemcpyAsync(L0.pb(), h.data(), L0.count * 8, cudaMemcpyHostToDevice, c.stream));
    MgBC bc = level_bc(c, 0, false);
    dim3 g, b; core_dims(L0, g, b);
    k_mg_init_p<double><<<g, b, 0, c.stream>>>(lview<double>(L0, L0.pa()), lcview<double>(L0, L0.pb()), bc);
    count_launch(c);
    std::vector<double> out(L0.count);
    SARAS_CUDA_TRY(cudaMemcpyAsync(out.data(), L0.pa(), L0.count * 8, cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    double m = 0;
    for (int i = -1; i <= X + 1; ++i) for (int j = -1; j <= Y + 1; ++j) for (int k = -1; k <= Z + 1; ++k) {
        int ng = (i < 0 || i > X) + (j < 0 || j > Y) + (k < 0 || k > Z);
        if (ng > 1) continue;
        m = std::max(m, std::fabs(out[v0.off(i, j, k)] - e[v0.off(i, j, k)]));
    }
    *err = m;
    return SARAS_OK;
}

}  // namespace saras
