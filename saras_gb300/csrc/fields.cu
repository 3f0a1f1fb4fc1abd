// fields.cu -- field operators, boundary fills, Crank-Nicolson Jacobi solves,
// projection and diagnostics of the SARAS time step on one GB300.
//
// Compiled with --fmad=false: every FP64 expression is rounded exactly as the
// reference writes it (no fused multiply-add contraction), which is what keeps
// the plain path within 1e-10 of the reference's CPU arithmetic.
//
// Uniform grids make every metric array a constant: xi_x = 1/L, xix2 =
// pow(1/L, 2), xixx = 0 (grid.cc:405-421).  Terms multiplied by xixx (= 0) are
// therefore omitted there; the remaining operations keep the reference's
// evaluation order.  On a stretched mesh (Mesh Type 'D' on some axis, the
// drop-in mode only) the reference-form kernels read the metric arrays at each
// point and evaluate the full expressions, xixx terms included.  Divisions by
// the grid spacings dXi = 2^-n and by hx*hx are exact power-of-two scalings and
// are applied as multiplications by the exact reciprocals.

#include <atomic>
#include <cmath>
#include <cstring>
#include <algorithm>

#include "context.cuh"
#include "df64.cuh"

namespace saras {

// ------------------------------------------------------------------ constants
// Constants of the split-FP64 Jacobi solve (see k_cn_delta).
struct CnDf {
    fpair kc[3];     // k1 c1, k1 c2, k1 c3 as float pairs (N0)
    float kf[3];     // the same as floats (the coupling sum of the sweeps)
    fpair invDn;     // 1 / Dn
};

struct UC {                 // stencil constants of one field
    double ih[3], ih2[3];   // 1/dXi and pow(1/dXi, 2)                 (derivative.cc:67-69)
    double h[3];            // dXi, dEt, dZt
    double m1[3];           // first-derivative metric xi_x = 1/L        (derivative.cc:77-105)
    double m2h[3];          // 0.5*xix2 (iScheme 1) or xix2              (derivative.cc:185-189)
    double gm[3];           // gradient / divergence metric 1/L          (sfield.cc:166-170)
    // stretched meshes (var != 0): the field's metric arrays along each axis
    // (x_Metric, xxMetric, x2Metric of derivative.cc:77-105), the collocated
    // xi_x of the gradient (sfield.cc:155-171) and the staggered xi_x of the
    // divergence (vfield.cc:299-320)
    const double *m1p[3], *mxp[3], *m2p[3], *gcp[3], *gsp[3];
    int var, half;          // half: iScheme 1 (the 0.5 of calcDerivative2xx)
    int planar;             // 2D: the y terms are left out (vfield.cc, sfield.cc under PLANAR)
};

static UC make_uc(const Ctx &c, int field) {
    UC u;
    const FieldInfo &f = c.info[field];
    for (int d = 0; d < 3; ++d) {
        u.ih[d] = c.ih[d];
        u.ih2[d] = c.ih2[d];
        u.h[d] = c.dXi[d];
        u.m1[d] = c.m1[d];
        u.m2h[d] = (c.p.iScheme == 1) ? 0.5 * c.m2[d] : c.m2[d];
        u.gm[d] = c.m1[d];
        const int st = f.stag[d] ? 1 : 0;
        u.m1p[d] = c.met[d][st][0];
        u.mxp[d] = c.met[d][st][1];
        u.m2p[d] = c.met[d][st][2];
        u.gcp[d] = c.met[d][0][0];
        u.gsp[d] = c.met[d][1][0];
    }
    u.var = c.stretched ? 1 : 0;
    u.half = c.p.iScheme == 1 ? 1 : 0;
    u.planar = c.planar ? 1 : 0;
    return u;
}

// metric of axis d at the point (i, j, k)
__device__ __forceinline__ double at_axis(const double *m, int d, int i, int j, int k) { return m[d == 0 ? i : d == 1 ? j : k]; }

template <typename T>
__device__ __forceinline__ void nbr(const View3<T> &F, int d, int i, int j, int k, double &fm, double &fp) {
    if (d == 0) { fm = F(i - 1, j, k); fp = F(i + 1, j, k); }
    else if (d == 1) { fm = F(i, j - 1, k); fp = F(i, j + 1, k); }
    else { fm = F(i, j, k - 1); fp = F(i, j, k + 1); }
}

// derivative::calcDerivative2xx (derivative.cc:178-191):
//   tmp = central12n(F)*ihx;  out = central22n(F)*ihx2;
//   result = xxMetric*tmp + 0.5*x2Metric*out   (uniform grid: 0.5*x2Metric*out)
__device__ __forceinline__ double d2_at(const View3<const double> &F, int d, int i, int j, int k, const UC &u) {
    double fm, fp, f0 = F(i, j, k);
    nbr(F, d, i, j, k, fm, fp);
    double out = (fm - 2.0 * f0 + fp) * u.ih2[d];
    if (!u.var) return u.m2h[d] * out;
    const double tmp = ((fp - fm) * 0.5) * u.ih[d];
    const double x2 = at_axis(u.m2p[d], d, i, j, k);
    return at_axis(u.mxp[d], d, i, j, k) * tmp + (u.half ? 0.5 * x2 * out : x2 * out);
}
// derivative::calcDerivative1_x (derivative.cc:121-126): x_Metric*(central12n(F)*ihx)
__device__ __forceinline__ double d1_at(const View3<const double> &F, int d, int i, int j, int k, const UC &u) {
    double fm, fp;
    nbr(F, d, i, j, k, fm, fp);
    double t = ((fp - fm) * 0.5) * u.ih[d];
    return (u.var ? at_axis(u.m1p[d], d, i, j, k) : u.m1[d]) * t;
}
// gradient metric (collocated xi_x along axis C) and divergence metric (staggered xi_x along d)
__device__ __forceinline__ double grad_m(const UC &u, int C, int i, int j, int k) { return u.var ? at_axis(u.gcp[C], C, i, j, k) : u.gm[C]; }
__device__ __forceinline__ double div_m(const UC &u, int d, int i, int j, int k) { return u.var ? at_axis(u.gsp[d], d, i, j, k) : u.gm[d]; }

// Interpolation slices (field.cc:309-575): interTemp(core) accumulated in
// slice order.  T = 0,1,2: target Vx, Vy, Vz;  T = 3: vertex field (P, T).
// S = source velocity component.
template <int T, int S> struct Slices;
#define SARAS_SLICE1(T_, S_)                                                                   \
    template <> struct Slices<T_, S_> {                                                        \
        static constexpr int n = 1;                                                            \
        __device__ static __forceinline__ double sum(const View3<const double> &V, int i, int j, int k) { \
            return V(i, j, k);                                                                 \
        }                                                                                      \
        __device__ static __forceinline__ fpair sump(const View3<const double> &V, int i, int j, int k) { \
            return fp_of(V(i, j, k));                                                          \
        }                                                                                      \
    };
#define SARAS_SLICE2(T_, S_, a, b, c)                                                          \
    template <> struct Slices<T_, S_> {                                                        \
        static constexpr int n = 2;                                                            \
        __device__ static __forceinline__ double sum(const View3<const double> &V, int i, int j, int k) { \
            return V(i, j, k) + V(i + (a), j + (b), k + (c));                                  \
        }                                                                                      \
        __device__ static __forceinline__ fpair sump(const View3<const double> &V, int i, int j, int k) { \
            return fp_add(fp_of(V(i, j, k)), fp_of(V(i + (a), j + (b), k + (c))));            \
        }                                                                                      \
    };
#define SARAS_SLICE4(T_, S_, a1, b1, c1, a2, b2, c2, a3, b3, c3)                                \
    template <> struct Slices<T_, S_> {                                                        \
        static constexpr int n = 4;                                                            \
        __device__ static __forceinline__ double sum(const View3<const double> &V, int i, int j, int k) { \
            return V(i, j, k) + V(i + (a1), j + (b1), k + (c1)) + V(i + (a2), j + (b2), k + (c2)) + \
                   V(i + (a3), j + (b3), k + (c3));                                             \
        }                                                                                      \
        __device__ static __forceinline__ fpair sump(const View3<const double> &V, int i, int j, int k) { \
            return fp_add(fp_add(fp_of(V(i, j, k)), fp_of(V(i + (a1), j + (b1), k + (c1)))),   \
                          fp_add(fp_of(V(i + (a2), j + (b2), k + (c2))), fp_of(V(i + (a3), j + (b3), k + (c3))))); \
        }                                                                                      \
    };
SARAS_SLICE1(0, 0)
SARAS_SLICE4(0, 1, 0, -1, 0, 1, 0, 0, 1, -1, 0)
SARAS_SLICE4(0, 2, 0, 0, -1, 1, 0, 0, 1, 0, -1)
SARAS_SLICE4(1, 0, -1, 0, 0, 0, 1, 0, -1, 1, 0)
SARAS_SLICE1(1, 1)
SARAS_SLICE4(1, 2, 0, 0, -1, 0, 1, 0, 0, 1, -1)
SARAS_SLICE4(2, 0, -1, 0, 0, 0, 0, 1, -1, 0, 1)
SARAS_SLICE4(2, 1, 0, -1, 0, 0, 0, 1, 0, -1, 1)
SARAS_SLICE1(2, 2)
SARAS_SLICE2(3, 0, -1, 0, 0)
SARAS_SLICE2(3, 1, 0, -1, 0)
SARAS_SLICE2(3, 2, 0, 0, -1)

template <int T, int S>
__device__ __forceinline__ double interp(const View3<const double> &V, int i, int j, int k) {
    return Slices<T, S>::sum(V, i, j, k);
}

struct Vel {
    View3<const double> v[3];
};

// H -= interTemp*derivTemp/size for the three directions (vfield.cc:163-253,
// sfield.cc:113-142).  Division by the slice count (1, 2 or 4) is exact.
template <int T>
__device__ __forceinline__ double nlin_update(double H, const View3<const double> &F, const Vel &V, int i, int j, int k, const UC &u) {
    H = H - (interp<T, 0>(V.v[0], i, j, k) * d1_at(F, 0, i, j, k, u)) * (1.0 / Slices<T, 0>::n);
    if (!u.planar) H = H - (interp<T, 1>(V.v[1], i, j, k) * d1_at(F, 1, i, j, k, u)) * (1.0 / Slices<T, 1>::n);
    H = H - (interp<T, 2>(V.v[2], i, j, k) * d1_at(F, 2, i, j, k, u)) * (1.0 / Slices<T, 2>::n);
    return H;
}

__device__ __forceinline__ double diff_sum(const View3<const double> &F, int i, int j, int k, const UC &u) {
    if (u.planar) return d2_at(F, 0, i, j, k, u) + d2_at(F, 2, i, j, k, u);
    return d2_at(F, 0, i, j, k, u) + d2_at(F, 1, i, j, k, u) + d2_at(F, 2, i, j, k, u);
}

// Thread -> point mapping over a box [lo, lo+ext) with k fastest.
struct Box {
    int lo[3], ext[3];
};
__device__ __forceinline__ bool box_point(const Box &b, int &i, int &j, int &k) {
    k = b.lo[2] + blockIdx.x * blockDim.x + threadIdx.x;
    j = b.lo[1] + blockIdx.y * blockDim.y + threadIdx.y;
    i = b.lo[0] + blockIdx.z * blockDim.z + threadIdx.z;
    return k < b.lo[2] + b.ext[2] && j < b.lo[1] + b.ext[1] && i < b.lo[0] + b.ext[0];
}
static void box_launch_dims(const Box &b, dim3 &grid, dim3 &block) {
    block = dim3(64, 4, 1);
    if (b.ext[2] <= 32) block = dim3(32, 8, 1);
    grid = dim3((b.ext[2] + block.x - 1) / block.x, (b.ext[1] + block.y - 1) / block.y, b.ext[0]);
}
static Box core_box(const FieldInfo &f) { Box b; for (int d = 0; d < 3; ++d) { b.lo[d] = 0; b.ext[d] = f.n[d]; } return b; }
static Box full_box(const FieldInfo &f) { Box b; for (int d = 0; d < 3; ++d) { b.lo[d] = -1; b.ext[d] = f.n[d] + 2; } return b; }

static View3<const double> cview(const Ctx &c, int field) {
    const FieldInfo &f = c.info[field];
    View3<const double> v;
    View3<double> w = make_view<double>(c.f[field], f.n[0], f.n[1], f.n[2]);
    v.p = w.p; v.n[0] = w.n[0]; v.n[1] = w.n[1]; v.n[2] = w.n[2]; v.sx = w.sx; v.sy = w.sy;
    return v;
}
static View3<double> mview(const Ctx &c, int field) {
    const FieldInfo &f = c.info[field];
    return make_view<double>(c.f[field], f.n[0], f.n[1], f.n[2]);
}
static View3<double> mview_ptr(const Ctx &c, int field, double *p) {
    const FieldInfo &f = c.info[field];
    return make_view<double>(p, f.n[0], f.n[1], f.n[2]);
}

// ------------------------------------------------------------------ operator kernels
// vfield::computeDiff / sfield::computeDiff: H(core) += d2xx; += d2yy; += d2zz.
__global__ void k_op_diff(View3<double> H, View3<const double> F, Box b, UC u) {
    int i, j, k;
    if (!box_point(b, i, j, k)) return;
    double h = H(i, j, k);
    h += d2_at(F, 0, i, j, k, u);
    if (!u.planar) h += d2_at(F, 1, i, j, k, u);
    h += d2_at(F, 2, i, j, k, u);
    H(i, j, k) = h;
}

template <int T>
__global__ void k_op_nlin(View3<double> H, View3<const double> F, Vel V, Box b, UC u) {
    int i, j, k;
    if (!box_point(b, i, j, k)) return;
    H(i, j, k) = nlin_update<T>(H(i, j, k), F, V, i, j, k, u);
}

// sfield::gradient (sfield.cc:155-171): G(core of component C) = m*(S(+e_C) - S)/dXi
template <int C>
__global__ void k_gradient(View3<double> G, View3<const double> S, Box b, UC u) {
    int i, j, k;
    if (!box_point(b, i, j, k)) return;
    double sp = C == 0 ? S(i + 1, j, k) : C == 1 ? S(i, j + 1, k) : S(i, j, k + 1);
    G(i, j, k) = (grad_m(u, C, i, j, k) * (sp - S(i, j, k))) * u.ih[C];
}

// vfield::divergence (vfield.cc:299-320), then optionally mgRHS *= 1/dt
// (hydro_d3.cc:326-327).  Writes the whole padded array (ghosts = 0).
// Folded per-axis factors of the fast forms (fastKernels = 1).
struct Fold3 {
    double k[3];
};

// fast != 0: the same divergence with gm * ih * scale folded into one factor
// per axis and the sum as fused multiply-adds (6 FP64 operations a point
// instead of 12; GB300's FP64 pipe, not HBM, bounds this kernel).
__global__ void k_divergence(View3<double> D, Vel V, Box full, UC u, double scale, int do_scale, int force_one, int fast,
                             Fold3 fk) {
    int i, j, k;
    if (!box_point(full, i, j, k)) return;
    double out = 0.0;
    if (force_one) { D(i, j, k) = 1.0; return; }
    if (i >= 0 && j >= 0 && k >= 0 && i < D.n[0] && j < D.n[1] && k < D.n[2]) {
        double dx = V.v[0](i, j, k) - V.v[0](i - 1, j, k);
        double dy = V.v[1](i, j, k) - V.v[1](i, j - 1, k);
        double dz = V.v[2](i, j, k) - V.v[2](i, j, k - 1);
        if (fast) {
            D(i, j, k) = fma(fk.k[0], dx, fma(fk.k[1], dy, fk.k[2] * dz));
            return;
        }
        double tx = (div_m(u, 0, i, j, k) * dx) * u.ih[0];
        double ty = (div_m(u, 1, i, j, k) * dy) * u.ih[1];
        double tz = (div_m(u, 2, i, j, k) * dz) * u.ih[2];
        out = u.planar ? tx + tz : tx + ty + tz;
    }
    if (do_scale) out = out * scale;
    D(i, j, k) = out;
}

// Split-FP64 form (fastKernels = 2) of the scaled divergence: the three face
// differences in FP64 (the velocity is nearly solenoidal, so the divergence is
// about 1e-10 of the velocity's scale and the differences need all 53 bits:
// split values of 47 bits leave 1e-5 of noise in the pressure right-hand
// side), each difference split into a float pair, the folded factors as float
// pairs, one FP64 addition per point; one thread per (j, k) column of the P
// full box marching along i with Vx(i-1) carried.  Points outside the P core
// are 0, as in k_divergence.
struct DivDf {
    fpair k[3];
};
constexpr int kProjMarch = 8;   // points per thread along i (divergence, projection)

__global__ void __launch_bounds__(256) k_divergence_df(View3<double> D, Vel V, Box full, DivDf q) {
    int k = full.lo[2] + blockIdx.x * 32 + threadIdx.x;
    int j = full.lo[1] + blockIdx.y * 8 + threadIdx.y;
    int i0 = full.lo[0] + blockIdx.z * kProjMarch;
    if (k >= full.lo[2] + full.ext[2] || j >= full.lo[1] + full.ext[1]) return;
    int iend = min(i0 + kProjMarch, full.lo[0] + full.ext[0]);
    bool jk = j >= 0 && k >= 0 && j < D.n[1] && k < D.n[2];
    double xm = 0.0;
    bool have = false;   // xm holds Vx(i-1)
    for (int i = i0; i < iend; ++i) {
        if (!(jk && i >= 0 && i < D.n[0])) { D(i, j, k) = 0.0; continue; }
        if (!have) { xm = V.v[0](i - 1, j, k); have = true; }
        double xc = V.v[0](i, j, k);
        fpair dx = fp_of(xc - xm);
        fpair dy = fp_of(V.v[1](i, j, k) - V.v[1](i, j - 1, k));
        fpair dz = fp_of(V.v[2](i, j, k) - V.v[2](i, j, k - 1));
        fpair sum = fp_fma(q.k[0], dx, fp_fma(q.k[1], dy, fp_mul(q.k[2], dz)));
        D(i, j, k) = f2d(sum.h) + f2d(sum.l);
        xm = xc;
    }
}

// Whole-array dst = a*dst + b*src (field arithmetic of field.cc:631-715).
__global__ void k_axpby(double *dst, double a, const double *src, double b, long n) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long stride = (long)gridDim.x * blockDim.x;
    for (; t < n; t += stride) {
        double x = dst[t];
        if (a != 1.0) x = a * x;
        if (src) x = x + b * src[t];
        dst[t] = x;
    }
}

// ------------------------------------------------------------------ fused NSE RHS
// hydro_d3::timeAdvance lines 259-295 for one component C at its core points:
//   H = 0; H += d2xx; H += d2yy; H += d2zz; H *= visc; H -= NL_x, NL_y, NL_z;
//   [Vz: H += Fb*avg(T)]; H -= grad P; H *= dt; H += V.
// nseRHS ghosts are never read (the Jacobi solve reads the bulk only).
struct RhsArgs {
    View3<double> H;
    View3<const double> F;   // the component itself
    Vel V;
    View3<const double> P;
    View3<const double> T;
    Box b;
    UC u;
    double visc, dt, Fb;
    int buoyancy;
};
template <int C>
__global__ void k_rhs(RhsArgs a) {
    int i, j, k;
    if (!box_point(a.b, i, j, k)) return;
    const UC &u = a.u;
    double h = diff_sum(a.F, i, j, k, u);
    h = h * a.visc;
    h = nlin_update<C>(h, a.F, a.V, i, j, k, u);
    if (C == 2 && a.buoyancy) {
        double t = (a.T(i, j, k) + a.T(i, j, k + 1)) * 0.5;
        h = h + a.Fb * t;
    }
    double sp = C == 0 ? a.P(i + 1, j, k) : C == 1 ? a.P(i, j + 1, k) : a.P(i, j, k + 1);
    double g = (grad_m(u, C, i, j, k) * (sp - a.P(i, j, k))) * u.ih[C];
    h = h - g;
    h = h * a.dt;
    h = h + a.F(i, j, k);
    a.H(i, j, k) = h;
}

// Fast form (fastKernels = 1) of the same right-hand side: constants folded,
// fused multiply-adds; not bit-identical to the reference order.
struct RhsFast {
    double K2[3];     // visc * m2h * ih2 (second derivatives)
    double K1[3];     // 0.5 * ih * m1 (first derivatives)
    double G[3];      // gm * ih (gradient)
    double Fb2;       // Fb / 2
    double dt;
};
template <int C>
__global__ void __launch_bounds__(256) k_rhs_fast(RhsArgs a, RhsFast q) {
    int i, j, k;
    if (!box_point(a.b, i, j, k)) return;
    const View3<const double> &F = a.F;
    double f0 = F(i, j, k);
    double sx = fma(-2.0, f0, F(i - 1, j, k) + F(i + 1, j, k));
    double sy = fma(-2.0, f0, F(i, j - 1, k) + F(i, j + 1, k));
    double sz = fma(-2.0, f0, F(i, j, k - 1) + F(i, j, k + 1));
    double h = fma(q.K2[0], sx, fma(q.K2[1], sy, q.K2[2] * sz));
    double dx = (F(i + 1, j, k) - F(i - 1, j, k)) * q.K1[0];
    double dy = (F(i, j + 1, k) - F(i, j - 1, k)) * q.K1[1];
    double dz = (F(i, j, k + 1) - F(i, j, k - 1)) * q.K1[2];
    h = fma(-interp<C, 0>(a.V.v[0], i, j, k), dx * (1.0 / Slices<C, 0>::n), h);
    h = fma(-interp<C, 1>(a.V.v[1], i, j, k), dy * (1.0 / Slices<C, 1>::n), h);
    h = fma(-interp<C, 2>(a.V.v[2], i, j, k), dz * (1.0 / Slices<C, 2>::n), h);
    if (C == 2 && a.buoyancy) h = fma(q.Fb2, a.T(i, j, k) + a.T(i, j, k + 1), h);
    double sp = C == 0 ? a.P(i + 1, j, k) : C == 1 ? a.P(i, j + 1, k) : a.P(i, j, k + 1);
    h = fma(-q.G[C], sp - a.P(i, j, k), h);
    a.H(i, j, k) = fma(h, q.dt, f0);
}

// Split-FP64 form (fastKernels = 2): k_rhs_df3 below, float-pair arithmetic
// (df64.cuh) from split values, every intermediate good to about 2^-44.

// All three components in one pass, written straight as the first iterate of
// the split-FP64 Jacobi solve.  With C0 = V at the start of the step the delta
// form's N0 = H - C0 + k1 sum_d c_d S_d(C0) (k_cn_pack) does not contain C0:
//   A = N0 / Dn = sum_d KL_d S_d - sum_d KN_d s_d delta_d - KG dP [+ KB (T + T')]
// with S_d = F(+d) + F(-d) - 2F, delta_d = F(+d) - F(-d), s_d the velocity
// values averaged along d (summed; the 1/count is in KN_d), and the constants
// KL_d = (dt visc m2h ih2 + k1 c_d) / Dn, KN_d = dt 0.5 ih m1 / count / Dn,
// KG = dt gm ih / Dn, KB = dt Fb / 2 / Dn folded on the host.  nseRHS itself
// (H = F + dt h) is not formed: the solve needs only A, so the FP64 additions
// that would carry F's 53 bits into H are not spent.  A is about dt |h| in
// size and good to about 2^-44 of its largest term.
//
// A stencil of one component reads about a dozen values of the four fields,
// and splitting each read into a float pair would cost about 35 splits a point
// over the three components.  Here a CTA owns a 32 (k) x 8 (j) tile of columns
// and marches kRhs3March planes along i; each plane of Vx, Vy, Vz and P on the
// tile plus a one-point halo is read once, split once and kept in shared
// memory (four rolling planes, so one barrier a plane), from where the three
// components' stencils read it.  Indices are logical (each field keeps its own
// core counts and strides); a component is evaluated where (i, j, k) is in its
// core.
constexpr int kRhs3March = 16;
constexpr int kR3K = 34, kR3N = 10 * kR3K;   // tile (8 x 32) + halo, per field and plane

struct Rhs3K {
    fpair kl[3];   // Laplacian: viscous term and the Jacobi coupling of N0
    fpair kn[3];   // advection
    fpair kg;      // pressure gradient
    fpair kb;      // buoyancy (Vz)
};

struct Rhs3Args {
    const double *f[4];        // Vx, Vy, Vz, P
    int n[4][3];               // their core counts
    long sx[4], sy[4];         // and strides
    const double *T;           // buoyancy: T, in P's layout
    float *n0h[3], *n0l[3];    // A of each component, component layouts
    int nu[3];                 // union of the cores
    int edgeK;                 // nu[2] - 1 when it is a multiple of 32 (the tiles then end below it), else -1
    int buoyancy;
    Rhs3K q[3];
};

// p + m - 2 c as an unnormalised pair: two TwoSums of the high parts (exact),
// the low parts and rounding errors in the second float.
__device__ __forceinline__ fpair lap_pair(fpair p, fpair m, fpair c) {
    float s, e, h, e2;
    two_sum(p.h, m.h, s, e);
    two_sum(s, -2.0f * c.h, h, e2);
    return fpair{h, e2 + (e + ((p.l + m.l) - 2.0f * c.l))};
}

// p - m as an unnormalised pair.
__device__ __forceinline__ fpair sub_pair(fpair p, fpair m) {
    float s, e;
    two_sum(p.h, -m.h, s, e);
    return fpair{s, e + (p.l - m.l)};
}

// a + b + c + d as an unnormalised pair.
__device__ __forceinline__ fpair sum4_pair(fpair a, fpair b, fpair c, fpair d) {
    float s1, e1, s2, e2, s, e3;
    two_sum(a.h, b.h, s1, e1);
    two_sum(c.h, d.h, s2, e2);
    two_sum(s1, s2, s, e3);
    return fpair{s, (e1 + e2 + e3) + ((a.l + b.l) + (c.l + d.l))};
}

// a + b + c as an unnormalised pair.
__device__ __forceinline__ fpair sum3_pair(fpair a, fpair b, fpair c) {
    float s1, e1, s, e2;
    two_sum(a.h, b.h, s1, e1);
    two_sum(s1, c.h, s, e2);
    return fpair{s, (e1 + e2) + ((a.l + b.l) + c.l)};
}

__device__ __forceinline__ fpair fp_scale(fpair a, float f) { return fpair{a.h * f, a.l * f}; }

// ISO: equal spacing and metrics on the three axes, where KL_0 = KL_1 = KL_2 and
// the advection constants are KN_C along the component's own axis and KN_C / 4
// (exactly: the same FP64 value divided by 4 before the split) for the two
// four-point averages, so the three Laplacians take one product and the three
// advection terms one more.  The sums are accumulated unnormalised and
// normalised once.
// G(f, di, dj, dk): field f at (i + di, j + dj, k + dk) as a float pair.
template <int C, bool ISO, class Get>
__device__ __forceinline__ void rhs3_point(const Rhs3Args &a, const Get &G, int i, int j, int k) {
    if (i >= a.n[C][0] || j >= a.n[C][1] || k >= a.n[C][2]) return;
    const long o = (long)(i + 1) * a.sx[C] + (long)(j + 1) * a.sy[C] + (k + 1);
    const Rhs3K &q = a.q[C];
    fpair c = G(C, 0, 0, 0), ex = G(C, 1, 0, 0), wx = G(C, -1, 0, 0);
    fpair ey = G(C, 0, 1, 0), wy = G(C, 0, -1, 0), ez = G(C, 0, 0, 1), wz = G(C, 0, 0, -1);
    fpair s0, s1, s2, dp;
    if (C == 0) {
        s0 = c;
        s1 = sum4_pair(G(1, 0, 0, 0), G(1, 0, -1, 0), G(1, 1, 0, 0), G(1, 1, -1, 0));
        s2 = sum4_pair(G(2, 0, 0, 0), G(2, 0, 0, -1), G(2, 1, 0, 0), G(2, 1, 0, -1));
        dp = sub_pair(G(3, 1, 0, 0), G(3, 0, 0, 0));
    } else if (C == 1) {
        s0 = sum4_pair(G(0, 0, 0, 0), G(0, 0, 1, 0), G(0, -1, 0, 0), G(0, -1, 1, 0));
        s1 = c;
        s2 = sum4_pair(G(2, 0, 0, 0), G(2, 0, 0, -1), G(2, 0, 1, 0), G(2, 0, 1, -1));
        dp = sub_pair(G(3, 0, 1, 0), G(3, 0, 0, 0));
    } else {
        s0 = sum4_pair(G(0, 0, 0, 0), G(0, 0, 0, 1), G(0, -1, 0, 0), G(0, -1, 0, 1));
        s1 = sum4_pair(G(1, 0, 0, 0), G(1, 0, -1, 0), G(1, 0, 0, 1), G(1, 0, -1, 1));
        s2 = c;
        dp = sub_pair(G(3, 0, 0, 1), G(3, 0, 0, 0));
    }
    const fpair d0 = sub_pair(ex, wx), d1 = sub_pair(ey, wy), d2 = sub_pair(ez, wz);
    fpair acc;
    if (ISO) {
        acc = fp_mul_u(q.kl[0], sum3_pair(lap_pair(ex, wx, c), lap_pair(ey, wy, c), lap_pair(ez, wz, c)));
        fpair adv;
        if (C == 0) adv = fp_fma_u(s0, d0, fp_scale(fp_fma_u(s1, d1, fp_mul_u(s2, d2)), 0.25f));
        else if (C == 1) adv = fp_fma_u(s1, d1, fp_scale(fp_fma_u(s0, d0, fp_mul_u(s2, d2)), 0.25f));
        else adv = fp_fma_u(s2, d2, fp_scale(fp_fma_u(s0, d0, fp_mul_u(s1, d1)), 0.25f));
        acc = fp_fma_u(fp_neg(q.kn[C]), adv, acc);
    } else {
        acc = fp_fma_u(q.kl[0], lap_pair(ex, wx, c), fp_fma_u(q.kl[1], lap_pair(ey, wy, c), fp_mul_u(q.kl[2], lap_pair(ez, wz, c))));
        acc = fp_fma_u(fp_neg(q.kn[0]), fp_mul_u(s0, d0), acc);
        acc = fp_fma_u(fp_neg(q.kn[1]), fp_mul_u(s1, d1), acc);
        acc = fp_fma_u(fp_neg(q.kn[2]), fp_mul_u(s2, d2), acc);
    }
    if (C == 2 && a.buoyancy) {
        long ot = (long)(i + 1) * a.sx[3] + (long)(j + 1) * a.sy[3] + (k + 1);
        acc = fp_fma_u(q.kb, fp_add(fp_of(a.T[ot]), fp_of(a.T[ot + 1])), acc);
    }
    acc = fp_fma_u(fp_neg(q.kg), dp, acc);
    acc = fp_norm(acc.h, acc.l);
    a.n0h[C][o] = acc.h;
    a.n0l[C][o] = acc.l;
}

template <bool ISO>
__global__ void __launch_bounds__(256, 5) k_rhs_df3(Rhs3Args a) {
    __shared__ float2 sm[4][4][kR3N];
    const int tid = threadIdx.y * 32 + threadIdx.x;
    if (a.edgeK >= 0 && blockIdx.x == gridDim.x - 1) {
        // the last column k = edgeK, (i, j) numbered j fastest, one point a thread
        // with its operands read from global memory (a 32-wide tile there would run
        // every warp's instructions for one active lane)
        const long t = ((long)blockIdx.z * gridDim.y + blockIdx.y) * 256 + tid;
        if (t >= (long)a.nu[0] * a.nu[1]) return;
        const int i = (int)(t / a.nu[1]), j = (int)(t - (long)i * a.nu[1]), k = a.edgeK;
        auto G = [&](int f, int di, int dj, int dk) -> fpair {
            return fp_of(a.f[f][(long)(i + di + 1) * a.sx[f] + (long)(j + dj + 1) * a.sy[f] + (k + dk + 1)]);
        };
        rhs3_point<0, ISO>(a, G, i, j, k);
        rhs3_point<1, ISO>(a, G, i, j, k);
        rhs3_point<2, ISO>(a, G, i, j, k);
        return;
    }
    const int k0 = blockIdx.x * 32, j0 = blockIdx.y * 8, i0 = blockIdx.z * kRhs3March;
    const int iend = min(i0 + kRhs3March, a.nu[0]);
    int js[2], ks[2];
    bool lt[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        int t = tid + 256 * s;
        int jj = t / kR3K;
        js[s] = j0 - 1 + jj;
        ks[s] = k0 - 1 + (t - jj * kR3K);
        lt[s] = t < kR3N;
    }
    auto load_plane = [&](int ip) {
        float2(*slot)[kR3N] = sm[ip & 3];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!lt[s]) continue;
            int t = tid + 256 * s, j = js[s], k = ks[s];
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                if (ip > a.n[f][0] || j > a.n[f][1] || k > a.n[f][2]) continue;   // outside the padded field
                fpair x = fp_of(a.f[f][(long)(ip + 1) * a.sx[f] + (long)(j + 1) * a.sy[f] + (k + 1)]);
                slot[f][t] = make_float2(x.h, x.l);
            }
        }
    };
    load_plane(i0 - 1);
    load_plane(i0);
    const int j = j0 + threadIdx.y, k = k0 + threadIdx.x;
    const int c0 = (threadIdx.y + 1) * kR3K + (threadIdx.x + 1);
    for (int i = i0; i < iend; ++i) {
        load_plane(i + 1);
        __syncthreads();
        auto G = [&](int f, int di, int dj, int dk) -> fpair {
            float2 v = sm[(i + di) & 3][f][c0 + dj * kR3K + dk];
            return fpair{v.x, v.y};
        };
        rhs3_point<0, ISO>(a, G, i, j, k);
        rhs3_point<1, ISO>(a, G, i, j, k);
        rhs3_point<2, ISO>(a, G, i, j, k);
    }
}

// The constants of every component have the isotropic form rhs3_point's ISO
// path assumes (bitwise: the same pairs, and a quarter of the own axis's
// advection constant on the other two).
static bool rhs3_iso(const Rhs3Args &a) {
    auto same = [](fpair x, fpair y) { return x.h == y.h && x.l == y.l; };
    for (int q = 0; q < 3; ++q) {
        const Rhs3K &k = a.q[q];
        if (!same(k.kl[0], k.kl[1]) || !same(k.kl[0], k.kl[2])) return false;
        for (int d = 0; d < 3; ++d)
            if (d != q && !same(k.kn[d], fpair{k.kn[q].h * 0.25f, k.kn[q].l * 0.25f})) return false;
    }
    return true;
}

static RhsFast make_rhs_fast(const Ctx &c, double visc) {
    RhsFast q;
    for (int d = 0; d < 3; ++d) {
        double m2h = (c.p.iScheme == 1) ? 0.5 * c.m2[d] : c.m2[d];
        q.K2[d] = visc * m2h * c.ih2[d];
        q.K1[d] = 0.5 * c.ih[d] * c.m1[d];
        q.G[d] = c.m1[d] * c.ih[d];
    }
    q.Fb2 = 0.5 * c.Fb;
    q.dt = c.dt;
    return q;
}

// scalar_d3::timeAdvance lines 344-355: tmpRHS for T (vertex field).
__global__ void k_trhs(RhsArgs a) {
    int i, j, k;
    if (!box_point(a.b, i, j, k)) return;
    const UC &u = a.u;
    double h = diff_sum(a.F, i, j, k, u);
    h = h * a.visc;
    h = nlin_update<3>(h, a.F, a.V, i, j, k, u);
    h = h * a.dt;
    h = h + a.F(i, j, k);
    a.H(i, j, k) = h;
}

// ------------------------------------------------------------------ boundary kernels
// Out-of-place application of a boundary program: out(p) = resolve(p) with
// base(q) = in(q).  Bulk points are copied when copy_bulk is set.
__global__ void k_bc_apply(View3<double> out, View3<const double> in, BcProgram prog, Box full, int copy_bulk) {
    int i, j, k;
    if (!box_point(full, i, j, k)) return;
    if (in_box(prog.blo, prog.bhi, i, j, k)) {
        if (copy_bulk) out(i, j, k) = in(i, j, k);
        return;
    }
    bool targeted = false;
    for (int o = 0; o < prog.nops; ++o) if (in_box(prog.op[o].lo, prog.op[o].hi, i, j, k)) { targeted = true; break; }
    if (!targeted) { if (copy_bulk) out(i, j, k) = in(i, j, k); return; }
    out(i, j, k) = bc_resolve(prog, i, j, k, [&](int a, int b, int c) -> double { return in(a, b, c); });
}

// Blocks a slab of the shell kernels (k_bc_apply_shell, k_cn_delta_shell,
// k_project_shell): each thread resolves boundary programs with dependent
// loads, so the slabs want many threads in flight (257^3: 256 blocks a slab
// took 0.187 ms a Jacobi solve and 0.279 ms a projection, against 0.191 and
// 0.289 with 64 and 0.192 and 0.289 with 1024).
constexpr int kShellBlocks = 256;

// k_bc_apply in place (copy_bulk = 0) over the non-bulk points only, as six
// disjoint slabs (blockIdx.y: along axis d = slab / 2 the points below / above
// the bulk range, the axes before d restricted to the bulk range, the axes
// after d full): the bulk points, which the in-place form leaves alone, cost no
// threads.
__global__ void k_bc_apply_shell(View3<double> out, View3<const double> in, BcProgram prog, Box full) {
    const int s = blockIdx.y, d = s >> 1;
    int lo[3], hi[3];
    for (int e = 0; e < 3; ++e) {
        if (e < d) { lo[e] = prog.blo[e]; hi[e] = prog.bhi[e]; }
        else { lo[e] = full.lo[e]; hi[e] = full.lo[e] + full.ext[e] - 1; }
    }
    if (s & 1) lo[d] = prog.bhi[d] + 1;
    else hi[d] = prog.blo[d] - 1;
    if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) return;
    const int n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1, n = (hi[0] - lo[0] + 1) * n1 * n2;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int r = t / n2, k = lo[2] + (t - r * n2), q = r / n1, j = lo[1] + (r - q * n1), i = lo[0] + q;
        bool targeted = false;
        for (int o = 0; o < prog.nops; ++o) if (in_box(prog.op[o].lo, prog.op[o].hi, i, j, k)) { targeted = true; break; }
        if (!targeted) continue;
        out(i, j, k) = bc_resolve(prog, i, j, k, [&](int a, int b, int c) -> double { return in(a, b, c); });
    }
}

// ------------------------------------------------------------------ Crank-Nicolson Jacobi
// hydro_d3::solveVx (hydro_d3.cc:374-422) fused: one launch computes the
// residual of the incoming iterate V_in over the bulk (lines 393-407) and the
// next iterate V_out = BCs(guess) over the whole padded box (lines 375-391),
// where guess is the Jacobi update on the bulk and 0 elsewhere.
struct CnArgs {
    View3<double> out;
    View3<const double> in;
    View3<const double> rhs;
    BcProgram prog;
    Box full;
    double c1, c2, c3;       // hy2hz2*xix2, hz2hx2*ety2, hx2hy2*ztz2
    double dt, X, coef, Dn;  // hydro: X = hx2hy2hz2*2*Re, Dn = 1 + dt*B/(Re*hx2hy2hz2)
    double iX, iDn;          // RN(1/X), RN(1/Dn): the divisions as div_rn
    int scalarForm;          // scalar_d3: ((A*dt)*coef)/X + rhs, Dn = 1 + (dt*coef)*B/h
    double lx, ly, lz;       // residual: metric * 1/(h*h)
    double resCoef;          // inverseRe (hydro) or nu / kappa (scalar)
    int withResidual;
    double *resMax;
    // stretched meshes: the metrics of the component at each index (mx(i),
    // my(j), mz(k) of hydro_d3.cc:378-400), so c1..c3, B, Dn and lx..lz are
    // formed per point from hy2hz2, hz2hx2, hx2hy2, h3 = hx2hy2hz2, Re, ihx2..ihz2
    const double *mx, *my, *mz;
    double hy2hz2, hz2hx2, hx2hy2, h3, Re, ihx2, ihy2, ihz2;
    int var;
    int planar;   // 2D (hydro_d2.cc:293-309): no y term in the update and the residual
};

__device__ __forceinline__ double cn_guess(const CnArgs &a, int i, int j, int k) {
    const View3<const double> &V = a.in;
    double c1 = a.c1, c2 = a.c2, c3 = a.c3, Dn = a.Dn;
    if (a.var) {
        c1 = a.hy2hz2 * a.mx[i];
        c2 = a.planar ? 0.0 : a.hz2hx2 * a.my[j];
        c3 = a.hx2hy2 * a.mz[k];
        const double B = a.planar ? c1 + c3 : c1 + c2 + c3;
        Dn = a.scalarForm ? 1.0 + a.dt * a.coef * B / a.h3 : 1.0 + a.dt * B / (a.Re * a.h3);
    }
    double A = a.planar ? c1 * (V(i + 1, j, k) + V(i - 1, j, k)) + c3 * (V(i, j, k + 1) + V(i, j, k - 1))
                        : c1 * (V(i + 1, j, k) + V(i - 1, j, k)) + c2 * (V(i, j + 1, k) + V(i, j - 1, k)) + c3 * (V(i, j, k + 1) + V(i, j, k - 1));
    double num = div_rn(a.scalarForm ? (A * a.dt) * a.coef : A * a.dt, a.X, a.iX);
    return a.var ? (num + a.rhs(i, j, k)) / Dn : div_rn(num + a.rhs(i, j, k), Dn, a.iDn);
}

__global__ void k_cn(CnArgs a) {
    int i, j, k;
    bool ok = box_point(a.full, i, j, k);
    double res = 0.0;
    if (ok) {
        bool bulk = in_box(a.prog.blo, a.prog.bhi, i, j, k);
        if (bulk) {
            if (a.withResidual) {
                const View3<const double> &V = a.in;
                double v0 = V(i, j, k);
                double L;
                if (a.planar && a.var)
                    L = (a.mx[i] * (V(i + 1, j, k) - 2.0 * v0 + V(i - 1, j, k))) * a.ihx2 +
                        (a.mz[k] * (V(i, j, k + 1) - 2.0 * v0 + V(i, j, k - 1))) * a.ihz2;
                else if (a.planar)
                    L = (a.lx * (V(i + 1, j, k) - 2.0 * v0 + V(i - 1, j, k))) + (a.lz * (V(i, j, k + 1) - 2.0 * v0 + V(i, j, k - 1)));
                else if (a.var)
                    L = (a.mx[i] * (V(i + 1, j, k) - 2.0 * v0 + V(i - 1, j, k))) * a.ihx2 +
                        (a.my[j] * (V(i, j + 1, k) - 2.0 * v0 + V(i, j - 1, k))) * a.ihy2 +
                        (a.mz[k] * (V(i, j, k + 1) - 2.0 * v0 + V(i, j, k - 1))) * a.ihz2;
                else
                    L = (a.lx * (V(i + 1, j, k) - 2.0 * v0 + V(i - 1, j, k))) +
                        (a.ly * (V(i, j + 1, k) - 2.0 * v0 + V(i, j - 1, k))) +
                        (a.lz * (V(i, j, k + 1) - 2.0 * v0 + V(i, j, k - 1)));
                double val = v0 - L * 0.5 * a.dt * a.resCoef;
                res = fabs(val - a.rhs(i, j, k));
                if (res != res) res = INFINITY;   // a NaN residual never converges
            }
            a.out(i, j, k) = cn_guess(a, i, j, k);
        } else {
            a.out(i, j, k) = bc_resolve(a.prog, i, j, k, [&](int x, int y, int z) -> double {
                return in_box(a.prog.blo, a.prog.bhi, x, y, z) ? cn_guess(a, x, y, z) : 0.0;
            });
        }
    }
    if (a.withResidual) block_max_to(res, a.resMax);
}

// Fast form of the same Jacobi iteration (fastKernels = 1): the two divisions
// become multiplications by precomputed reciprocals and the sums are fused
// multiply-adds.  The residual of the input C, C - k2 Lap(C) - rhs, equals
// Dn (C - J(C)) for the Jacobi image J(C) = (rhs + k2 offdiag(C)) / Dn, so the
// kernel reports max |C - J(C)| and the host multiplies by Dn: no second
// stencil evaluation.  Same fixed point and stopping rule, not bit-identical.
struct CnFast {
    View3<double> out;
    View3<const double> in, rhs;
    BcProgram prog;
    Box full;
    double c1, c2, c3, k1, invDn;   // guess = fma(A, k1, rhs) * invDn
    int withResidual;
    double *resMax;                 // max |C - guess| (times Dn on the host)
};

__device__ __forceinline__ double cn_guess_fast(const CnFast &a, int i, int j, int k) {
    const View3<const double> &V = a.in;
    double A = fma(a.c1, V(i + 1, j, k) + V(i - 1, j, k), fma(a.c2, V(i, j + 1, k) + V(i, j - 1, k), a.c3 * (V(i, j, k + 1) + V(i, j, k - 1))));
    return fma(A, a.k1, a.rhs(i, j, k)) * a.invDn;
}

__global__ void __launch_bounds__(256) k_cn_fast(CnFast a) {
    int i, j, k;
    bool ok = box_point(a.full, i, j, k);
    double res = 0.0;
    if (ok) {
        if (in_box(a.prog.blo, a.prog.bhi, i, j, k)) {
            const View3<const double> &V = a.in;
            double C = V(i, j, k);
            double ew = V(i + 1, j, k) + V(i - 1, j, k), ns = V(i, j + 1, k) + V(i, j - 1, k), ud = V(i, j, k + 1) + V(i, j, k - 1);
            double A = fma(a.c1, ew, fma(a.c2, ns, a.c3 * ud));
            double o = fma(A, a.k1, a.rhs(i, j, k)) * a.invDn;
            a.out(i, j, k) = o;
            if (a.withResidual) res = C - o;   // |.| and NaN ordering in block_max_to (integer pipe)
        } else {
            a.out(i, j, k) = bc_resolve(a.prog, i, j, k, [&](int x, int y, int z) -> double {
                return in_box(a.prog.blo, a.prog.bhi, x, y, z) ? cn_guess_fast(a, x, y, z) : 0.0;
            });
        }
    }
    if (a.withResidual) block_max_to(res, a.resMax);
}

// Split-FP64 form of the same Jacobi iteration (fastKernels = 2), in delta
// form.  With Dn = 1 + 2 k1 (c1 + c2 + c3) the Jacobi image of an iterate C is
//   J(C) = C + corr,  corr = (rhs - C + k1 (c1 S_x(C) + c2 S_y(C) + c3 S_z(C))) / Dn,
// S_d(C) = C(+d) + C(-d) - 2C.  Writing C = C0 + D for the field C0 at the
// start of the solve,
//   corr = (N0 - D + k1 sum_d c_d S_d(D)) / Dn,  N0 = rhs - C0 + k1 sum_d c_d S_d(C0),
// so N0 is formed once per solve (k_cn_pack, float-pair arithmetic from split
// FP64 values) and every sweep (k_cn_delta) works on the small correction D,
// held as a float pair: the sweep reads and writes 8 bytes per point like the
// FP64 form but does no FP64 arithmetic at all, and k_cn_unpack forms
// C0 + D in FP64 at the end, so C0 keeps all its bits.  Accuracy: about 2^-44
// of the largest of |rhs|, |C0| in N0, and of |D| in the sweeps (the Jacobi
// tolerance is 1e-8).  Boundary points: the field's boundary program resolved
// on C0 + D in float pairs (constant -> value, copy -> copy, reflect -> 2c - v),
// then minus C0 there, as the FP64 form resolves it on C.
static CnDf cn_df_consts(const CnFast &fa) {
    CnDf d;
    auto pr = [](double x) { fpair r; r.h = (float)x; r.l = (float)(x - (double)r.h); return r; };
    d.kc[0] = pr(fa.k1 * fa.c1);
    d.kc[1] = pr(fa.k1 * fa.c2);
    d.kc[2] = pr(fa.k1 * fa.c3);
    for (int q = 0; q < 3; ++q) d.kf[q] = d.kc[q].h;
    d.invDn = pr(fa.invDn);
    return d;
}

// A = N0 / Dn at the bulk points of the field's full box.
__global__ void __launch_bounds__(256) k_cn_pack(View3<const double> V, View3<const double> rhs, BcProgram prog, Box full, CnDf f,
                                                 float *n0h, float *n0l) {
    int i, j, k;
    if (!box_point(full, i, j, k) || !in_box(prog.blo, prog.bhi, i, j, k)) return;
    fpair c = fp_of(V(i, j, k)), c2 = fpair{-2.0f * c.h, -2.0f * c.l};
    fpair sx = fp_add(fp_add(fp_of(V(i + 1, j, k)), fp_of(V(i - 1, j, k))), c2);
    fpair sy = fp_add(fp_add(fp_of(V(i, j + 1, k)), fp_of(V(i, j - 1, k))), c2);
    fpair sz = fp_add(fp_add(fp_of(V(i, j, k + 1)), fp_of(V(i, j, k - 1))), c2);
    fpair q = fp_add(fp_add(fp_mul(f.kc[0], sx), fp_mul(f.kc[1], sy)), fp_mul(f.kc[2], sz));
    fpair n = fp_add(fp_of(rhs(i, j, k) - V(i, j, k)), q);   // rhs - C0 in FP64: both O(1), the difference small
    n = fp_mul(n, f.invDn);                                  // stored as A = N0 / Dn (the first sweep from D = 0)
    long o = V.off(i, j, k);
    n0h[o] = n.h;
    n0l[o] = n.l;
}

struct CnDelta {
    const double *C0;
    const float *n0h, *n0l;
    const float *dh, *dl;      // D in
    float *oh, *ol;            // D out
    long sx, sy;               // strides of the padded layout (k stride 1)
    BcProgram prog;
    Box full;
    CnDf f;
    int withResidual;
    double *resMax;            // max |corr| (times Dn on the host)
    double *vout;              // final sweep: C0 + D out into this FP64 array instead of D
    __device__ long off(int i, int j, int k) const { return (long)(i + 1) * sx + (long)(j + 1) * sy + (k + 1); }
};

// The new iterate of point o: D out, or (final sweep) C0 + D in FP64, the sum
// k_cn_unpack forms.
template <bool FINAL>
__device__ __forceinline__ void cn_delta_store(const CnDelta &a, long o, fpair out) {
    if (FINAL) {
        a.vout[o] = (a.C0[o] + f2d(out.h)) + f2d(out.l);
    } else {
        a.oh[o] = out.h;
        a.ol[o] = out.l;
    }
}

// p + m - 2 c for float pairs p, m, c (one axis of the discrete Laplacian of
// D) as a float: the high parts' sum by TwoSum, its difference with 2 c.h
// (exact for smooth D, where the two are within a factor of two), then the
// rounding error and the low parts.  The pressure right-hand side is the
// divergence of the Jacobi result, about 1e-10 of the velocity's scale, and the
// plain float sum of the high parts (24 bits of D) left 1e-5 of noise in it;
// this form keeps the sum to 24 bits of itself.
__device__ __forceinline__ float cn_lap1(fpair p, fpair m, fpair c) {
    float s, e;
    two_sum(p.h, m.h, s, e);
    return (s - 2.0f * c.h) + (e + ((p.l + m.l) - 2.0f * c.l));
}

// The Jacobi update of D at bulk point o from its neighbours along each axis:
// corr = (N0 - D + sum_d k1 c_d (p_d + m_d - 2 D)) / Dn, with A = N0 / Dn stored
// (the first iterate from D = 0, which the right-hand-side kernel writes).
__device__ __forceinline__ fpair cn_delta_update(const CnDelta &a, long o, fpair D, fpair xp, fpair xm, fpair yp, fpair ym, fpair zp,
                                                 fpair zm, fpair &corr) {
    float q = fmaf(a.f.kf[0], cn_lap1(xp, xm, D), fmaf(a.f.kf[1], cn_lap1(yp, ym, D), a.f.kf[2] * cn_lap1(zp, zm, D)));
    corr = fp_fma(fp_add(fpair{q, 0.0f}, fp_neg(D)), a.f.invDn, fpair{a.n0h[o], a.n0l[o]});
    return fp_add(D, corr);
}

__device__ __forceinline__ fpair cn_d(const CnDelta &a, long o) { return fpair{a.dh[o], a.dl[o]}; }

// D + corr at bulk point o.
__device__ __forceinline__ fpair cn_delta_image(const CnDelta &a, long o, fpair &corr) {
    return cn_delta_update(a, o, cn_d(a, o), cn_d(a, o + a.sx), cn_d(a, o - a.sx), cn_d(a, o + a.sy), cn_d(a, o - a.sy), cn_d(a, o + 1),
                           cn_d(a, o - 1), corr);
}

__device__ __forceinline__ fpair fp_of_c(double x) {
    fpair r;
    r.h = __double2float_rn(x);
    r.l = __double2float_rn(x - (double)r.h);
    return r;
}

// Boundary point (i, j, k): the program resolved on C0 + D in float pairs (the
// FP64 form's bc_resolve with base = Jacobi image at bulk points, 0 elsewhere),
// minus C0 there.  A chain of copies (periodic images, no reflection or
// constant) gives D(source) + (C0(source) - C0(here)): exactly D(source) when
// C0 holds exact copies there, so the field's copied ghosts stay exact copies
// of their sources, as the FP64 form's are.
template <bool COPY>
__device__ __forceinline__ fpair cn_delta_boundary(const CnDelta &a, int i, int j, int k, long o) {
    const BcProgram &prog = a.prog;
    int chain[kMaxBcOps];
    int nchain = 0;
    fpair value = fpair{0.0f, 0.0f};
    bool haveConst = false, reflects = false;
    int q[3] = {i, j, k};
    for (int op = prog.nops - 1; op >= 0; --op) {
        const BcOp &b = prog.op[op];
        if (q[0] < b.lo[0] || q[0] > b.hi[0] || q[1] < b.lo[1] || q[1] > b.hi[1] || q[2] < b.lo[2] || q[2] > b.hi[2]) continue;
        if (b.kind == OP_CONST) { value = fp_of_c(b.c); haveConst = true; break; }
        chain[nchain++] = op;
        reflects = reflects || b.kind == OP_REFLECT;
        q[0] += b.shift[0]; q[1] += b.shift[1]; q[2] += b.shift[2];
    }
    if (!haveConst && in_box(prog.blo, prog.bhi, q[0], q[1], q[2])) {
        long os = a.off(q[0], q[1], q[2]);
        fpair corr;
        fpair d = COPY ? cn_d(a, os) : cn_delta_image(a, os, corr);
        if (!reflects) {
            fpair z = fp_add(fp_of(a.C0[os]), fp_neg(fp_of(a.C0[o])));
            return (z.h == 0.0f && z.l == 0.0f) ? d : fp_add(d, z);
        }
        value = fp_add(fp_of(a.C0[os]), d);
    }
    for (int cix = nchain - 1; cix >= 0; --cix) {
        const BcOp &b = prog.op[chain[cix]];
        if (b.kind == OP_REFLECT) value = fp_add(fp_of_c(2.0 * b.c), fp_neg(value));
    }
    return fp_add(value, fp_neg(fp_of(a.C0[o])));
}

// One thread per (j, k) column of the full box, marching kCnMarch points
// along i: the index work is paid once per column segment.  kCnColumns: the
// columns numbered k fastest over the whole (j, k) plane, 256 a block
// (blockIdx.y the segment), else 32 x 8 tiles (blockIdx.z the segment), which
// leave the last tile of each 259-point row with three active lanes a warp
// (the final sweep: 189 us in columns against 192 in tiles at 257^3).
// Segment length and blocks an SM, measured on the final sweep at 257^3: 4
// points with six blocks (40 registers) 159 us, 4 with five 163, 8 with four
// 171, 16 with three 197.
constexpr int kCnMarch = 4;
constexpr bool kCnColumns = true;

template <bool FINAL>
__global__ void __launch_bounds__(256, 6) k_cn_delta(CnDelta a) {
    int k, j, i0;
    bool on;
    if (kCnColumns) {
        const int W = a.full.ext[2], t = blockIdx.x * 256 + threadIdx.x, jj = t / W;
        j = a.full.lo[1] + jj;
        k = a.full.lo[2] + (t - jj * W);
        i0 = a.full.lo[0] + blockIdx.y * kCnMarch;
        on = jj < a.full.ext[1];
    } else {
        k = a.full.lo[2] + blockIdx.x * 32 + threadIdx.x;
        j = a.full.lo[1] + blockIdx.y * 8 + threadIdx.y;
        i0 = a.full.lo[0] + blockIdx.z * kCnMarch;
        on = k < a.full.lo[2] + a.full.ext[2] && j < a.full.lo[1] + a.full.ext[1];
    }
    unsigned m = 0u;
    if (on) {
        int iend = min(i0 + kCnMarch, a.full.lo[0] + a.full.ext[0]);
        bool bulkJK = j >= a.prog.blo[1] && j <= a.prog.bhi[1] && k >= a.prog.blo[2] && k <= a.prog.bhi[2];
        if (bulkJK && iend == i0 + kCnMarch && i0 >= a.prog.blo[0] && iend - 1 <= a.prog.bhi[0]) {
            // a whole segment of bulk points: branch-free, the column's own i-1 / i / i+1
            // values carried in registers, and every store after the segment's last
            // load (the output arrays may alias the inputs as far as the compiler
            // can tell, so a store between loads would hold the later loads back)
            const long o = a.off(i0, j, k);
            fpair dm = cn_d(a, o - a.sx), dc = cn_d(a, o);
            fpair out[kCnMarch];
            double v[kCnMarch];
#pragma unroll
            for (int q = 0; q < kCnMarch; ++q) {
                const long oq = o + q * a.sx;
                fpair dp = cn_d(a, oq + a.sx);
                fpair corr;
                out[q] = cn_delta_update(a, oq, dc, dp, dm, cn_d(a, oq + a.sy), cn_d(a, oq - a.sy), cn_d(a, oq + 1), cn_d(a, oq - 1), corr);
                if (FINAL) v[q] = (a.C0[oq] + f2d(out[q].h)) + f2d(out[q].l);
                m = max(m, __float_as_uint(corr.h) & 0x7fffffffu);
                dm = dc;
                dc = dp;
            }
#pragma unroll
            for (int q = 0; q < kCnMarch; ++q) {
                const long oq = o + q * a.sx;
                if (FINAL) a.vout[oq] = v[q];
                else { a.oh[oq] = out[q].h; a.ol[oq] = out[q].l; }
            }
            iend = i0;   // segment done (the generic loop below runs no iteration)
        }
        for (int i = i0; i < iend; ++i) {
            if (!(bulkJK && i >= a.prog.blo[0] && i <= a.prog.bhi[0])) continue;   // boundary points: k_cn_delta_shell
            long o = a.off(i, j, k);
            fpair corr;
            fpair out = cn_delta_image(a, o, corr);
            m = max(m, __float_as_uint(corr.h) & 0x7fffffffu);   // |corr| bits; NaN stays above Inf
            cn_delta_store<FINAL>(a, o, out);
        }
    }
    if (a.withResidual) block_maxf_to(__uint_as_float(m), a.resMax);
}

// The non-bulk points of the full box (the boundary program's targets), as six
// disjoint slabs: along axis d the points below / above the bulk range, with the
// axes before d restricted to the bulk range and the axes after d full.
// COPY: no Jacobi update -- the non-bulk points of D (in place in dh / dl)
// from the current D at their sources: the boundary values of the first
// iterate A, which the right-hand-side kernel writes on the bulk only.
template <bool FINAL, bool COPY>
__global__ void k_cn_delta_shell(CnDelta a) {
    int s = blockIdx.y, d = s >> 1;
    int lo[3], hi[3];
    for (int e = 0; e < 3; ++e) {
        if (e < d) { lo[e] = a.prog.blo[e]; hi[e] = a.prog.bhi[e]; }
        else { lo[e] = a.full.lo[e]; hi[e] = a.full.lo[e] + a.full.ext[e] - 1; }
    }
    if (s & 1) lo[d] = a.prog.bhi[d] + 1;
    else hi[d] = a.prog.blo[d] - 1;
    if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) return;
    // 32-bit index arithmetic: a slab holds fewer than 2^31 points
    const int n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1, n = (hi[0] - lo[0] + 1) * n1 * n2;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int r = t / n2, k = lo[2] + (t - r * n2), q = r / n1, j = lo[1] + (r - q * n1), i = lo[0] + q;
        long o = a.off(i, j, k);
        cn_delta_store<FINAL>(a, o, cn_delta_boundary<COPY>(a, i, j, k, o));
    }
}

// C0 + D in FP64 over the whole padded array (in place on the field).
__global__ void k_cn_unpack(double *V, const float *dh, const float *dl, long n) {
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        V[t] = (V[t] + f2d(dh[t])) + f2d(dl[t]);
}

// ------------------------------------------------------------------ projection
// hydro_d3.cc:357-367: V -= dt*grad(Pp) on the component core (gradient = 0
// elsewhere), optionally followed by the component's boundary program.
// FAST (fastKernels = 1): V - fastDt * (Pp(+1) - Pp) as one fused
// multiply-add, fastDt = gm * ih * dt folded on the host.
template <int C, bool FAST>
__global__ void k_project(View3<double> out, View3<const double> in, View3<const double> Pp, BcProgram prog, Box full,
                          UC u, double dt, int with_bc, double fastDt) {
    int i, j, k;
    if (!box_point(full, i, j, k)) return;
    auto base = [&](int x, int y, int z) -> double {
        double v = in(x, y, z);
        if (x >= 0 && y >= 0 && z >= 0 && x < in.n[0] && y < in.n[1] && z < in.n[2]) {
            double sp = C == 0 ? Pp(x + 1, y, z) : C == 1 ? Pp(x, y + 1, z) : Pp(x, y, z + 1);
            if (FAST) return fma(-fastDt, sp - Pp(x, y, z), v);
            double g = (grad_m(u, C, x, y, z) * (sp - Pp(x, y, z))) * u.ih[C];
            v = v - g * dt;
        }
        return v;
    };
    if (!with_bc || in_box(prog.blo, prog.bhi, i, j, k)) { out(i, j, k) = base(i, j, k); return; }
    bool targeted = false;
    for (int o = 0; o < prog.nops; ++o) if (in_box(prog.op[o].lo, prog.op[o].hi, i, j, k)) { targeted = true; break; }
    out(i, j, k) = targeted ? bc_resolve(prog, i, j, k, base) : base(i, j, k);
}

// The fused-form projection with its boundary program split in two launches
// (as the split Jacobi sweep): k_project_bulk marches the bulk box (the points
// no boundary op targets: V - fastDt (Pp(+1) - Pp), no device calls, Pp along
// the component's own axis carried in registers for Vx), k_project_shell
// resolves the program on the remaining points of the full box.
template <int C>
__global__ void __launch_bounds__(256) k_project_bulk(View3<double> out, View3<const double> in, View3<const double> Pp, BcProgram prog,
                                                      double fastDt) {
    // one thread per (j, k) column of the bulk, numbered k fastest over the
    // whole bulk plane (256 a block, blockIdx.y the segment): 32-wide tiles
    // would leave warps with one active lane on rows of 2^m + 1 points, which
    // still occupy the FP64 pipe
    const int W = prog.bhi[2] - prog.blo[2] + 1, t = blockIdx.x * 256 + threadIdx.x, jj = t / W;
    int k = prog.blo[2] + (t - jj * W);
    int j = prog.blo[1] + jj;
    int i0 = prog.blo[0] + blockIdx.y * kProjMarch;
    if (j > prog.bhi[1]) return;
    int iend = min(i0 + kProjMarch - 1, prog.bhi[0]);
    bool jk = j < in.n[1] && k < in.n[2];
    double pc = Pp(i0, j, k);
    for (int i = i0; i <= iend; ++i) {
        double v = in(i, j, k);
        double pn = C == 0 ? Pp(i + 1, j, k) : C == 1 ? Pp(i, j + 1, k) : Pp(i, j, k + 1);
        if (jk && i < in.n[0]) v = fma(-fastDt, pn - pc, v);
        out(i, j, k) = v;
        pc = C == 0 ? pn : Pp(i + 1, j, k);
    }
}

template <int C>
__global__ void k_project_shell(View3<double> out, View3<const double> in, View3<const double> Pp, BcProgram prog, Box full,
                                double fastDt) {
    int s = blockIdx.y, d = s >> 1;
    int lo[3], hi[3];
    for (int e = 0; e < 3; ++e) {
        if (e < d) { lo[e] = prog.blo[e]; hi[e] = prog.bhi[e]; }
        else { lo[e] = full.lo[e]; hi[e] = full.lo[e] + full.ext[e] - 1; }
    }
    if (s & 1) lo[d] = prog.bhi[d] + 1;
    else hi[d] = prog.blo[d] - 1;
    if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) return;
    auto base = [&](int x, int y, int z) -> double {
        double v = in(x, y, z);
        if (x >= 0 && y >= 0 && z >= 0 && x < in.n[0] && y < in.n[1] && z < in.n[2]) {
            double sp = C == 0 ? Pp(x + 1, y, z) : C == 1 ? Pp(x, y + 1, z) : Pp(x, y, z + 1);
            v = fma(-fastDt, sp - Pp(x, y, z), v);
        }
        return v;
    };
    // 32-bit index arithmetic: a slab holds fewer than 2^31 points
    const int n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1, n = (hi[0] - lo[0] + 1) * n1 * n2;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int r = t / n2, k = lo[2] + (t - r * n2), q = r / n1, j = lo[1] + (r - q * n1), i = lo[0] + q;
        bool targeted = false;
        for (int o = 0; o < prog.nops; ++o) if (in_box(prog.op[o].lo, prog.op[o].hi, i, j, k)) { targeted = true; break; }
        out(i, j, k) = targeted ? bc_resolve(prog, i, j, k, base) : base(i, j, k);
    }
}

// ------------------------------------------------------------------ diagnostics
// tseries::writeTSData (tseries.cc:137-246): per-block partial sums of the
// face-averaged energy and of <w T>, and the block max of the divergence over
// the collocated core range.
__global__ void k_diag(Vel V, View3<const double> T, int has_t, int nP0, int nP1, int nP2, int nc0, int nc1, int nc2,
                       UC u, double dv, double *partE, double *partU, double *partD) {
    __shared__ double se[32], su[32], sd[32];
    long n = (long)nP0 * nP1 * nP2;
    double e = 0.0, w = 0.0, dmax = -INFINITY;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        int k = (int)(t % nP2);
        int j = (int)((t / nP2) % nP1);
        int i = (int)(t / ((long)nP2 * nP1));
        double a = (V.v[0](i - 1, j, k) + V.v[0](i, j, k)) / 2.0;
        double b = (V.v[1](i, j - 1, k) + V.v[1](i, j, k)) / 2.0;
        double c = (V.v[2](i, j, k - 1) + V.v[2](i, j, k)) / 2.0;
        // tseries.cc:150-165: the cell volume from the collocated metrics (2D: x and z, tseries.cc:149-156)
        const double dvp = u.planar ? (u.h[0] / u.gcp[0][i]) * (u.h[2] / u.gcp[2][k])
                           : u.var  ? (u.h[0] / u.gcp[0][i]) * (u.h[1] / u.gcp[1][j]) * (u.h[2] / u.gcp[2][k])
                                    : dv;
        e += (u.planar ? a * a + c * c : a * a + b * b + c * c) * dvp;
        if (has_t) w += ((V.v[2](i, j, k) + V.v[2](i, j, k - 1)) / 2.0) * T(i, j, k) * dvp;
        if (i < nc0 && j < nc1 && k < nc2) {
            double tx = (div_m(u, 0, i, j, k) * (V.v[0](i, j, k) - V.v[0](i - 1, j, k))) * u.ih[0];
            double ty = (div_m(u, 1, i, j, k) * (V.v[1](i, j, k) - V.v[1](i, j - 1, k))) * u.ih[1];
            double tz = (div_m(u, 2, i, j, k) * (V.v[2](i, j, k) - V.v[2](i, j, k - 1))) * u.ih[2];
            dmax = fmax(dmax, u.planar ? tx + tz : tx + ty + tz);
        }
    }
    e = warp_sum(e); w = warp_sum(w); dmax = warp_max(dmax);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { se[wid] = e; su[wid] = w; sd[wid] = dmax; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double E = 0, U = 0, D = -INFINITY;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { E += se[q]; U += su[q]; D = fmax(D, sd[q]); }
        partE[blockIdx.x] = E; partU[blockIdx.x] = U; partD[blockIdx.x] = D;
    }
}

// Deterministic final reduction of per-block partials (fixed order).
__global__ void k_final_reduce(const double *part, int n, int op, double *out) {
    __shared__ double s[256];
    double acc = op == 0 ? 0.0 : -INFINITY;
    for (int t = threadIdx.x; t < n; t += blockDim.x) acc = op == 0 ? acc + part[t] : fmax(acc, part[t]);
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] = op == 0 ? s[threadIdx.x] + s[threadIdx.x + w] : fmax(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

// ------------------------------------------------------------------ host side
static void add_op(BcProgram &pg, int kind, const int lo[3], const int hi[3], const int sh[3], double cst) {
    if (pg.nops >= kMaxBcOps) return;   // at most 4 faces + 4 edges + 6 walls are ever added
    BcOp &o = pg.op[pg.nops++];
    o.kind = kind; o.c = cst;
    for (int d = 0; d < 3; ++d) { o.lo[d] = lo[d]; o.hi[d] = hi[d]; o.shift[d] = sh[d]; }
}

// mpidata::syncData at np = 1 (mpidata.cc:82-306): periodic faces over the
// core range of the other axes, then the four x-y edges over the core z range.
static void add_sync_ops(BcProgram &pg, const FieldInfo &f, bool xPer, bool yPer, bool planar) {
    int cx = f.n[0], cy = f.n[1], cz = f.n[2];
    int lx = f.stag[0] ? 1 : 0, hx = cx - 1 - (f.stag[0] ? 1 : 0);
    int ly = f.stag[1] ? 1 : 0, hy = cy - 1 - (f.stag[1] ? 1 : 0);
    if (xPer) {
        int lo[3] = {-1, 0, 0}, hi[3] = {-1, cy - 1, cz - 1}, sh[3] = {hx + 1, 0, 0};
        add_op(pg, OP_COPY, lo, hi, sh, 0);
        int lo2[3] = {cx, 0, 0}, hi2[3] = {cx, cy - 1, cz - 1}, sh2[3] = {lx - cx, 0, 0};
        add_op(pg, OP_COPY, lo2, hi2, sh2, 0);
    }
    if (planar) return;   // 2D: no y and no edge neighbours (parallel.cc:118-130, hydro.cc:188-191)
    if (yPer) {
        int lo[3] = {0, -1, 0}, hi[3] = {cx - 1, -1, cz - 1}, sh[3] = {0, hy + 1, 0};
        add_op(pg, OP_COPY, lo, hi, sh, 0);
        int lo2[3] = {0, cy, 0}, hi2[3] = {cx - 1, cy, cz - 1}, sh2[3] = {0, ly - cy, 0};
        add_op(pg, OP_COPY, lo2, hi2, sh2, 0);
    }
    int e1lo[3] = {-1, -1, 0}, e1hi[3] = {-1, -1, cz - 1}, e1s[3] = {hx + 1, hy + 1, 0};
    int e2lo[3] = {-1, cy, 0}, e2hi[3] = {-1, cy, cz - 1}, e2s[3] = {hx + 1, ly - cy, 0};
    int e3lo[3] = {cx, -1, 0}, e3hi[3] = {cx, -1, cz - 1}, e3s[3] = {lx - cx, hy + 1, 0};
    int e4lo[3] = {cx, cy, 0}, e4hi[3] = {cx, cy, cz - 1}, e4s[3] = {lx - cx, ly - cy, 0};
    add_op(pg, OP_COPY, e1lo, e1hi, e1s, 0);
    add_op(pg, OP_COPY, e2lo, e2hi, e2s, 0);
    add_op(pg, OP_COPY, e3lo, e3hi, e3s, 0);
    add_op(pg, OP_COPY, e4lo, e4hi, e4s, 0);
}

enum WallKind { W_DIR_CC, W_DIR_FC, W_NEU, W_PER_CC, W_PER_FC };
struct Wall { WallKind k; int wall; double v; };

// Wall objects of the boundary classes (lib/boundary/*.cc) as plane ops.
static void add_wall_op(BcProgram &pg, const FieldInfo &f, const Wall &w) {
    int dim = w.wall / 2;
    bool even = (w.wall % 2) == 0;
    int shiftVal = even ? 1 : -1;
    int w0 = f.blo[dim] - 1, w1 = f.bhi[dim] + 1;
    int windex = even ? w0 : w1;
    int lo[3] = {-1, -1, -1}, hi[3] = {f.n[0], f.n[1], f.n[2]};
    lo[dim] = hi[dim] = windex;
    int sh[3] = {0, 0, 0};
    switch (w.k) {
    case W_DIR_CC: add_op(pg, OP_CONST, lo, hi, sh, w.v); break;                          // dirichletCC.cc:71-75
    case W_DIR_FC: sh[dim] = shiftVal; add_op(pg, OP_REFLECT, lo, hi, sh, w.v); break;    // dirichletFC.cc:71-75
    case W_NEU: sh[dim] = shiftVal; add_op(pg, OP_COPY, lo, hi, sh, 0); break;           // neumannCC/FC
    case W_PER_CC: sh[dim] = (even ? w1 - 2 : w0 + 2) - windex; add_op(pg, OP_COPY, lo, hi, sh, 0); break;  // periodicCC.cc:72-83
    case W_PER_FC: sh[dim] = (even ? w1 - 1 : w0 + 1) - windex; add_op(pg, OP_COPY, lo, hi, sh, 0); break;  // periodicFC.cc:72-81
    }
}

// hydro::initVBC (hydro.cc:287-371) and scalar::initTBC (scalar.cc:185-227), in
// the order imposeU/V/W/TBCs apply them: Lft, Rgt, Frn, Bak, Top, Bot.
static std::vector<Wall> walls_for(const saras_params &p, int field, bool planar) {
    std::vector<Wall> w;
    // 2D: no front and back walls, no Vy boundary objects (hydro.cc:298-301, 320-353, scalar.cc:197-200)
    auto add = [&](WallKind k, int wall, double v) { if (!(planar && wall / 2 == 1)) w.push_back(Wall{k, wall, v}); };
    if (planar && field == SARAS_FIELD_VY) return w;
    if (field == SARAS_FIELD_VX) {
        if (!p.xPer) { if (p.probType == 3) { add(W_DIR_FC, 0, 1.0); add(W_NEU, 1, 0.0); } else { add(W_DIR_FC, 0, 0.0); add(W_DIR_FC, 1, 0.0); } }
        if (!p.yPer) { add(W_DIR_CC, 2, 0.0); add(W_DIR_CC, 3, 0.0); }
        if (p.zPer) { add(W_PER_CC, 5, 0); add(W_PER_CC, 4, 0); }
        else if (p.probType == 1) { add(W_DIR_CC, 5, 1.0); add(W_DIR_CC, 4, 0.0); }
        else { add(W_DIR_CC, 5, 0.0); add(W_DIR_CC, 4, 0.0); }
    } else if (field == SARAS_FIELD_VY) {
        if (!p.xPer) { if (p.probType == 3) { add(W_DIR_CC, 0, 0.0); add(W_NEU, 1, 0.0); } else { add(W_DIR_CC, 0, 0.0); add(W_DIR_CC, 1, 0.0); } }
        if (!p.yPer) { add(W_DIR_FC, 2, 0.0); add(W_DIR_FC, 3, 0.0); }
        if (p.zPer) { add(W_PER_CC, 5, 0); add(W_PER_CC, 4, 0); }
        else { add(W_DIR_CC, 5, 0.0); add(W_DIR_CC, 4, 0.0); }
    } else if (field == SARAS_FIELD_VZ) {
        if (!p.xPer) { if (p.probType == 3) { add(W_DIR_CC, 0, 0.0); add(W_NEU, 1, 0.0); } else { add(W_DIR_CC, 0, 0.0); add(W_DIR_CC, 1, 0.0); } }
        if (!p.yPer) { add(W_DIR_CC, 2, 0.0); add(W_DIR_CC, 3, 0.0); }
        if (p.zPer) { add(W_PER_FC, 5, 0); add(W_PER_FC, 4, 0); }
        else { add(W_DIR_FC, 5, 0.0); add(W_DIR_FC, 4, 0.0); }
    } else if (field == SARAS_FIELD_T) {
        if (!p.xPer) {
            if (p.probType == 5 || p.probType == 6 || p.probType == 8) { add(W_NEU, 0, 0.0); add(W_NEU, 1, 0.0); }
            else if (p.probType == 7) { add(W_DIR_CC, 0, 1.0); add(W_DIR_CC, 1, 0.0); }
        }
        if (!p.yPer) { add(W_NEU, 2, 0.0); add(W_NEU, 3, 0.0); }
        if (p.zPer) { add(W_PER_CC, 5, 0); add(W_PER_CC, 4, 0); }
        else if (p.probType == 5 || p.probType == 8) { add(W_DIR_CC, 5, 0.0); add(W_DIR_CC, 4, 1.0); }
        else if (p.probType == 6) { add(W_DIR_CC, 5, 1.0); add(W_DIR_CC, 4, 0.0); }
    }
    return w;
}

static void set_field_info(Ctx &c, int field, bool xs, bool ys, bool zs) {
    FieldInfo &f = c.info[field];
    bool st[3] = {xs, ys, zs};
    bool per[3] = {c.p.xPer != 0, c.p.yPer != 0, c.p.zPer != 0};
    for (int d = 0; d < 3; ++d) {
        f.stag[d] = st[d];
        f.n[d] = st[d] ? c.Ns[d] : c.Nc[d];
        f.blo[d] = 0; f.bhi[d] = f.n[d] - 1;
        if (st[d] && !per[d]) { f.blo[d] += 1; f.bhi[d] -= 1; }   // field.cc:206-219
    }
    if (c.planar) { f.blo[1] = 0; f.bhi[1] = 0; }                  // field.cc:221-224
    f.full.nops = 0; f.sync.nops = 0;
    add_sync_ops(f.sync, f, per[0], per[1], c.planar);
    add_sync_ops(f.full, f, per[0], per[1], c.planar);
    for (const Wall &w : walls_for(c.p, field, c.planar)) add_wall_op(f.full, f, w);
    for (int d = 0; d < 3; ++d) {
        f.full.blo[d] = f.sync.blo[d] = f.blo[d];
        f.full.bhi[d] = f.sync.bhi[d] = f.bhi[d];
    }
    // The sync program never targets core points; its "bulk" is the whole core.
    for (int d = 0; d < 3; ++d) { f.sync.blo[d] = 0; f.sync.bhi[d] = f.n[d] - 1; }
}

// Coordinates and metrics (grid.cc:290-320 defaults, createUniformGrid
// grid.cc:370-422, createTanHypGrid grid.cc:442-519): every axis is first
// uniform over its whole padded range; an axis with Mesh Type 'D' (xGrid = 2)
// then gets the double-sided tangent-hyperbolic map, with stretching factor
// "X/Y/Z Beta", on its core points (ghost entries keep the uniform values).
// The expressions are the reference's, so host code computing them must not
// contract multiplies and adds (the library is built with -ffp-contract=off).
static int grid_metrics(Ctx &c) {
    const saras_params &p = c.p;
    const int gtype[3] = {p.xGrid, p.yGrid, p.zGrid};
    const double beta[3] = {p.betaX, p.betaY, p.betaZ};
    c.stretched = false;
    size_t total = 0;
    for (int d = 0; d < 3; ++d) {
        const double Ld = c.L[d];
        const int n[2] = {c.Nc[d], c.Ns[d]};   // core counts: collocated, staggered
        auto xi = [&](int i) { return double(i) * c.dXi[d]; };   // grid.cc:333-352
        for (int st = 0; st < 2; ++st) {
            const int len = n[st] + 2;   // indices -1 .. n
            for (int m = 0; m < 3; ++m) c.hmet[d][st][m].assign(len, m == 0 ? c.m1[d] : m == 1 ? 0.0 : c.m2[d]);
            c.hcoord[d][st].assign(len, 0.0);
            for (int i = -1; i < n[st] + 1; ++i)
                c.hcoord[d][st][i + 1] = st ? Ld * xi(i) : Ld * (xi(i) + xi(i + 1)) / 2.0;
            total += 3 * (size_t)len;
        }
        if (c.planar && d == 1) {   // grid.cc:300-320: y coordinates keep their default 1
            for (int st = 0; st < 2; ++st) std::fill(c.hcoord[1][st].begin(), c.hcoord[1][st].end(), 1.0);
            continue;
        }
        if (gtype[d] != 2) continue;
        c.stretched = true;
        const double b = beta[d];
        for (int st = 0; st < 2; ++st) {
            for (int i = 0; i < n[st]; ++i) {
                const double x = st ? Ld * (1.0 - std::tanh(b * (1.0 - 2.0 * xi(i))) / std::tanh(b)) / 2.0
                                    : Ld * (1.0 - std::tanh(b * (1.0 - (xi(i) + xi(i + 1)))) / std::tanh(b)) / 2.0;
                c.hcoord[d][st][i + 1] = x;
                const double m1 = std::tanh(b) / (b * Ld * (1.0 - std::pow((1.0 - 2.0 * x / Ld) * std::tanh(b), 2)));
                c.hmet[d][st][0][i + 1] = m1;
                c.hmet[d][st][1][i + 1] = -4.0 * std::pow(std::tanh(b), 3) * (1.0 - 2.0 * x / Ld) /
                                          (b * Ld * Ld * std::pow(1.0 - std::pow(std::tanh(b) * (1.0 - 2.0 * x / Ld), 2), 2));
                c.hmet[d][st][2][i + 1] = std::pow(m1, 2.0);
            }
        }
    }
    SARAS_CUDA_TRY(cudaMalloc(&c.dmet, sizeof(double) * total));
    size_t off = 0;
    for (int d = 0; d < 3; ++d)
        for (int st = 0; st < 2; ++st)
            for (int m = 0; m < 3; ++m) {
                const std::vector<double> &h = c.hmet[d][st][m];
                SARAS_CUDA_TRY(cudaMemcpy(c.dmet + off, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
                c.met[d][st][m] = c.dmet + off + 1;
                off += h.size();
            }
    return SARAS_OK;
}

int fields_setup(Ctx &c) {
    const saras_params &p = c.p;
    int ind[3] = {p.xInd, p.yInd, p.zInd};
    double L[3] = {p.Lx, p.Ly, p.Lz};
    c.planar = p.yInd == 0;
    if (c.planar) L[1] = 1.0;                                   // grid.cc:88-92: yLen = dEt = 1
    for (int d = 0; d < 3; ++d) {
        c.Ns[d] = int(std::pow(2, ind[d])) + 1;                 // grid.cc:155-164
        c.Nc[d] = c.Ns[d] - 1;
        c.dXi[d] = 1.0 / double(c.Ns[d] - 1);                   // grid.cc:84-86
        if (c.planar && d == 1) { c.Ns[1] = 1; c.Nc[1] = 1; c.dXi[1] = 1.0; }   // grid.cc:183-188, 232-234
        c.ih[d] = 1.0 / c.dXi[d];                               // derivative.cc:67-69
        c.ih2[d] = std::pow(c.ih[d], 2.0);
        c.L[d] = L[d];
        c.m1[d] = 1.0 / L[d];                                   // grid.cc:405-421
        c.m2[d] = std::pow(c.m1[d], 2.0);
    }
    c.scalar = p.probType >= 5;
    c.inverseRe = 1.0 / p.Re;
    if (c.scalar) {
        if (p.rbcType == 1) { c.nu = p.Pr; c.kappa = 1.0; }
        else if (p.rbcType == 2) { c.nu = std::sqrt(p.Pr / p.Ra); c.kappa = 1.0 / std::sqrt(p.Pr * p.Ra); }
        else if (p.rbcType == 3) { c.nu = 1.0; c.kappa = 1.0 / p.Pr; }
        else { c.nu = std::sqrt(p.Pr / p.Ra); c.kappa = 1.0 / std::sqrt(p.Pr * p.Ra); }
        switch (p.rbcType) { case 1: c.Fb = p.Ra * p.Pr; break; case 2: c.Fb = 1.0; break; case 3: c.Fb = p.Ra; break; default: c.Fb = p.Pr; }
    } else { c.nu = 0; c.kappa = 0; c.Fb = 0; }
    c.dt = p.tStp;
    c.hz2hx2 = std::pow(c.dXi[2], 2.0) * std::pow(c.dXi[0], 2.0);   // hydro.cc:223-241
    c.hx2hy2 = std::pow(c.dXi[0], 2.0) * std::pow(c.dXi[1], 2.0);
    c.hy2hz2 = std::pow(c.dXi[1], 2.0) * std::pow(c.dXi[2], 2.0);
    c.hx2hy2hz2 = std::pow(c.dXi[0], 2.0) * std::pow(c.dXi[1], 2.0) * std::pow(c.dXi[2], 2.0);
    c.maxIterations = c.Nc[0] * c.Nc[1] * c.Nc[2];                  // hydro.cc:74
    if (int e = grid_metrics(c)) return e;
    c.totalVol = 0.0;                                                 // tseries.cc:90-108
    const double *wx = c.hmet[0][0][0].data() + 1, *wy = c.hmet[1][0][0].data() + 1, *wz = c.hmet[2][0][0].data() + 1;
    for (int iX = 0; iX < c.Ns[0]; iX++) for (int iY = 0; iY < c.Ns[1]; iY++) for (int iZ = 0; iZ < c.Ns[2]; iZ++)
        c.totalVol += c.planar ? (c.dXi[0] / wx[iX]) * (c.dXi[2] / wz[iZ])   // tseries.cc:93-99
                               : (c.dXi[0] / wx[iX]) * (c.dXi[1] / wy[iY]) * (c.dXi[2] / wz[iZ]);

    set_field_info(c, SARAS_FIELD_VX, false, true, true);
    set_field_info(c, SARAS_FIELD_VY, true, false, true);
    set_field_info(c, SARAS_FIELD_VZ, true, true, false);
    set_field_info(c, SARAS_FIELD_P, true, true, true);
    set_field_info(c, SARAS_FIELD_T, true, true, true);
    c.info[SARAS_FIELD_PP] = c.info[SARAS_FIELD_P];
    c.info[SARAS_FIELD_MGRHS] = c.info[SARAS_FIELD_P];
    c.info[SARAS_FIELD_TRHS] = c.info[SARAS_FIELD_T];
    c.info[SARAS_FIELD_NSE_X] = c.info[SARAS_FIELD_VX];
    c.info[SARAS_FIELD_NSE_Y] = c.info[SARAS_FIELD_VY];
    c.info[SARAS_FIELD_NSE_Z] = c.info[SARAS_FIELD_VZ];
    c.info[SARAS_FIELD_GRAD_X] = c.info[SARAS_FIELD_VX];
    c.info[SARAS_FIELD_GRAD_Y] = c.info[SARAS_FIELD_VY];
    c.info[SARAS_FIELD_GRAD_Z] = c.info[SARAS_FIELD_VZ];
    for (int fld = 0; fld < SARAS_NUM_FIELDS; ++fld) {
        const FieldInfo &f = c.info[fld];
        size_t bytes = sizeof(double) * (size_t)(f.n[0] + 2) * (f.n[1] + 2) * (f.n[2] + 2);
        SARAS_CUDA_TRY(cudaMalloc(&c.f[fld], bytes));
        SARAS_CUDA_TRY(cudaMemsetAsync(c.f[fld], 0, bytes, c.stream));
    }
    const int sf[4] = {SARAS_FIELD_VX, SARAS_FIELD_VY, SARAS_FIELD_VZ, SARAS_FIELD_T};
    for (int q = 0; q < 4; ++q) {
        const FieldInfo &f = c.info[sf[q]];
        size_t bytes = sizeof(double) * (size_t)(f.n[0] + 2) * (f.n[1] + 2) * (f.n[2] + 2);
        SARAS_CUDA_TRY(cudaMalloc(&c.scratch[q], bytes));
        SARAS_CUDA_TRY(cudaMemsetAsync(c.scratch[q], 0, bytes, c.stream));
    }
    // per-block partials of the reductions: one per column block and segment of
    // the finest level (k_tgt_stats), one per 4096-point chunk of a padded level
    {
        const long cols = (long)c.Ns[1] * c.Ns[2], pts = (long)(c.Ns[0] + 2) * (c.Ns[1] + 2) * (c.Ns[2] + 2);
        const long need = std::max((cols + 255) / 256 * ((c.Ns[0] + 3) / 4 + 1), pts / 4096 + 1);
        c.redCap = (int)std::max<long>(1 << 16, need);
    }
    SARAS_CUDA_TRY(cudaMalloc(&c.red, sizeof(double) * c.redCap * 3));
    SARAS_CUDA_TRY(cudaMalloc(&c.dscal, sizeof(double) * 64));
    SARAS_CUDA_TRY(cudaMalloc(&c.dflag, sizeof(int) * 16));
    SARAS_CUDA_TRY(cudaMallocHost(&c.hscal, sizeof(double) * 64));
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal, 0, sizeof(double) * 64, c.stream));
    return SARAS_OK;
}

static int check_launch(Ctx &c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { c.err = std::string(what) + ": " + cudaGetErrorString(e); return SARAS_CUDA_ERROR; }
    return SARAS_OK;
}

static int scratch_slot(int field) {
    switch (field) { case SARAS_FIELD_VX: return 0; case SARAS_FIELD_VY: return 1; case SARAS_FIELD_VZ: return 2; case SARAS_FIELD_T: return 3; }
    return -1;
}

// Out-of-place program application: scratch = BC(field), then swap buffers.
static int apply_program(Ctx &c, int field, const BcProgram &prog) {
    int slot = scratch_slot(field);
    const FieldInfo &f = c.info[field];
    Box fb = full_box(f);
    dim3 g, b;
    box_launch_dims(fb, g, b);
    if (slot >= 0) {
        k_bc_apply<<<g, b, 0, c.stream>>>(mview_ptr(c, field, c.scratch[slot]), cview(c, field), prog, fb, 1);
        count_launch(c);
        std::swap(c.f[field], c.scratch[slot]);
    } else {
        // Programs of fields without a scratch partner only copy from core
        // points that no op targets (syncData), so they run in place, on the
        // non-bulk points alone.
        k_bc_apply_shell<<<dim3(kShellBlocks, 6), 256, 0, c.stream>>>(mview(c, field), cview(c, field), prog, fb);
        count_launch(c);
    }
    return check_launch(c, "k_bc_apply");
}

int apply_bc(Ctx &c, int field) {
    if (field == SARAS_FIELD_T && !c.scalar) return SARAS_BAD_ARG;
    if (scratch_slot(field) < 0) return SARAS_BAD_ARG;
    return apply_program(c, field, c.info[field].full);
}

int sync_field(Ctx &c, int field) {
    if (field < 0 || field >= SARAS_NUM_FIELDS) return SARAS_BAD_ARG;
    return apply_program(c, field, c.info[field].sync);
}

static Vel make_vel(const Ctx &c) {
    Vel v;
    v.v[0] = cview(c, SARAS_FIELD_VX);
    v.v[1] = cview(c, SARAS_FIELD_VY);
    v.v[2] = cview(c, SARAS_FIELD_VZ);
    return v;
}

int vfield_compute_diff(Ctx &c) {
    for (int q = 0; q < 3; ++q) {
        if (c.planar && q == 1) continue;   // 2D: Vy takes no part (vfield.cc:119-131)
        UC u = make_uc(c, SARAS_FIELD_VX + q);
        Box b = core_box(c.info[SARAS_FIELD_VX + q]);
        dim3 g, bl; box_launch_dims(b, g, bl);
        k_op_diff<<<g, bl, 0, c.stream>>>(mview(c, SARAS_FIELD_NSE_X + q), cview(c, SARAS_FIELD_VX + q), b, u);
        count_launch(c);
    }
    return check_launch(c, "computeDiff");
}

int vfield_compute_nlin(Ctx &c) {
    Vel V = make_vel(c);
    for (int q = 0; q < 3; ++q) {
        if (c.planar && q == 1) continue;
        UC u = make_uc(c, SARAS_FIELD_VX + q);
        Box b = core_box(c.info[SARAS_FIELD_VX + q]);
        dim3 g, bl; box_launch_dims(b, g, bl);
        if (q == 0) k_op_nlin<0><<<g, bl, 0, c.stream>>>(mview(c, SARAS_FIELD_NSE_X), cview(c, SARAS_FIELD_VX), V, b, u);
        if (q == 1) k_op_nlin<1><<<g, bl, 0, c.stream>>>(mview(c, SARAS_FIELD_NSE_Y), cview(c, SARAS_FIELD_VY), V, b, u);
        if (q == 2) k_op_nlin<2><<<g, bl, 0, c.stream>>>(mview(c, SARAS_FIELD_NSE_Z), cview(c, SARAS_FIELD_VZ), V, b, u);
        count_launch(c);
    }
    return check_launch(c, "computeNLin");
}

int tfield_compute_diff(Ctx &c) {
    if (!c.scalar) return SARAS_BAD_ARG;
    UC u = make_uc(c, SARAS_FIELD_T);
    Box b = core_box(c.info[SARAS_FIELD_T]);
    dim3 g, bl; box_launch_dims(b, g, bl);
    k_op_diff<<<g, bl, 0, c.stream>>>(mview(c, SARAS_FIELD_TRHS), cview(c, SARAS_FIELD_T), b, u);
    count_launch(c);
    return check_launch(c, "T.computeDiff");
}

int tfield_compute_nlin(Ctx &c) {
    if (!c.scalar) return SARAS_BAD_ARG;
    UC u = make_uc(c, SARAS_FIELD_T);
    Box b = core_box(c.info[SARAS_FIELD_T]);
    dim3 g, bl; box_launch_dims(b, g, bl);
    k_op_nlin<3><<<g, bl, 0, c.stream>>>(mview(c, SARAS_FIELD_TRHS), cview(c, SARAS_FIELD_T), make_vel(c), b, u);
    count_launch(c);
    return check_launch(c, "T.computeNLin");
}

int sfield_gradient(Ctx &c, int sf) {
    if (sf != SARAS_FIELD_P && sf != SARAS_FIELD_PP) return SARAS_BAD_ARG;
    UC u = make_uc(c, SARAS_FIELD_P);
    for (int q = 0; q < 3; ++q) {
        if (c.planar && q == 1) continue;   // sfield.cc:167-169
        Box b = core_box(c.info[SARAS_FIELD_VX + q]);
        dim3 g, bl; box_launch_dims(b, g, bl);
        View3<double> G = mview(c, SARAS_FIELD_GRAD_X + q);
        if (q == 0) k_gradient<0><<<g, bl, 0, c.stream>>>(G, cview(c, sf), b, u);
        if (q == 1) k_gradient<1><<<g, bl, 0, c.stream>>>(G, cview(c, sf), b, u);
        if (q == 2) k_gradient<2><<<g, bl, 0, c.stream>>>(G, cview(c, sf), b, u);
        count_launch(c);
    }
    return check_launch(c, "gradient");
}

int vfield_divergence(Ctx &c, double *dst, bool scale_dt) {
    UC u = make_uc(c, SARAS_FIELD_P);
    Box fb = full_box(c.info[SARAS_FIELD_P]);
    dim3 g, bl; box_launch_dims(fb, g, bl);
    View3<double> D = mview_ptr(c, SARAS_FIELD_MGRHS, dst ? dst : c.f[SARAS_FIELD_MGRHS]);
    prof_begin(c, PK_DIVERGENCE, 0);
    Fold3 fk;
    for (int d = 0; d < 3; ++d) fk.k[d] = u.gm[d] * u.ih[d] * (scale_dt ? 1.0 / c.dt : 1.0);
    if (c.p.fastKernels == 2 && !(scale_dt && c.p.testPoisson)) {
        DivDf q;
        for (int d = 0; d < 3; ++d) { q.k[d].h = (float)fk.k[d]; q.k[d].l = (float)(fk.k[d] - (double)q.k[d].h); }
        dim3 gd((fb.ext[2] + 31) / 32, (fb.ext[1] + 7) / 8, (fb.ext[0] + kProjMarch - 1) / kProjMarch);
        k_divergence_df<<<gd, dim3(32, 8), 0, c.stream>>>(D, make_vel(c), fb, q);
    } else {
        k_divergence<<<g, bl, 0, c.stream>>>(D, make_vel(c), fb, u, 1.0 / c.dt, scale_dt ? 1 : 0,
                                             (scale_dt && c.p.testPoisson) ? 1 : 0, c.p.fastKernels != 0, fk);
    }
    count_launch(c);
    prof_end(c, PK_DIVERGENCE, 0, 5.0 * 8.0 * (double)D.size());
    return check_launch(c, "divergence");
}

int axpby(Ctx &c, int dst, double a, int src, double b) {
    if (dst < 0 || dst >= SARAS_NUM_FIELDS || src >= SARAS_NUM_FIELDS) return SARAS_BAD_ARG;
    long n = make_view<double>(c.f[dst], c.info[dst].n[0], c.info[dst].n[1], c.info[dst].n[2]).size();
    if (src >= 0) {
        long m = make_view<double>(c.f[src], c.info[src].n[0], c.info[src].n[1], c.info[src].n[2]).size();
        if (m != n) return SARAS_BAD_ARG;
    }
    int blocks = (int)std::min<long>((n + 255) / 256, 152L * 16);
    k_axpby<<<blocks, 256, 0, c.stream>>>(c.f[dst], a, src >= 0 ? c.f[src] : nullptr, b, n);
    count_launch(c);
    return check_launch(c, "axpby");
}

// Constants of the Jacobi solve of component comp (hydro_d3.cc:370-533,
// scalar_d3.cc:373-591): the reference form in a, the fused forms in fa.
static void cn_setup(Ctx &c, int comp, CnArgs &a, CnFast &fa) {
    int field = comp == 3 ? SARAS_FIELD_T : SARAS_FIELD_VX + comp;
    int rhsField = comp == 3 ? SARAS_FIELD_TRHS : SARAS_FIELD_NSE_X + comp;
    const FieldInfo &f = c.info[field];
    a.rhs = cview(c, rhsField);
    a.prog = f.full;
    a.full = full_box(f);
    // Metrics: every component's xix2/ety2/ztz2 equal pow(1/L,2) on uniform grids
    // (the T solve's ztz2Colloc of scalar_d3.cc:551,570 has the same value).
    // In 2D (dEt = 1) hy2hz2, hx2hy2 and hx2hy2hz2 equal the 2D coefficients hz2,
    // hx2 and hz2hx2 exactly (hydro.cc:225-232); the y term is left out.
    double xix2 = c.m2[0], ety2 = c.m2[1], ztz2 = c.m2[2];
    a.c1 = c.hy2hz2 * xix2;
    a.c2 = c.planar ? 0.0 : c.hz2hx2 * ety2;
    a.c3 = c.hx2hy2 * ztz2;
    double B = c.planar ? c.hy2hz2 * xix2 + c.hx2hy2 * ztz2 : (c.hy2hz2 * xix2 + c.hz2hx2 * ety2) + c.hx2hy2 * ztz2;
    a.dt = c.dt;
    if (!c.scalar) {
        a.scalarForm = 0;
        a.coef = 0;
        a.X = c.hx2hy2hz2 * 2.0 * c.p.Re;
        a.Dn = 1.0 + c.dt * B / (c.p.Re * c.hx2hy2hz2);
        a.iX = 1.0 / a.X;
        a.iDn = 1.0 / a.Dn;
        a.resCoef = c.inverseRe;
    } else {
        double coef = comp == 3 ? c.kappa : c.nu;
        a.scalarForm = 1;
        a.coef = coef;
        a.X = c.hx2hy2hz2 * 2.0;
        a.Dn = 1.0 + c.dt * coef * B / c.hx2hy2hz2;
        a.iX = 1.0 / a.X;
        a.iDn = 1.0 / a.Dn;
        a.resCoef = coef;
    }
    // residual: metric*(...)/(h*h); h*h is a power of two, so /(h*h) == *(1/(h*h))
    a.lx = xix2 * (1.0 / (c.dXi[0] * c.dXi[0]));
    a.ly = ety2 * (1.0 / (c.dXi[1] * c.dXi[1]));
    a.lz = ztz2 * (1.0 / (c.dXi[2] * c.dXi[2]));
    a.resMax = c.dscal;
    // the metrics of the component (hydro_d3.cc:378-400, 433-455, 488-510;
    // the T solve's ztz2Colloc, scalar_d3.cc:549-571)
    static const int kSt[4][3] = {{0, 1, 1}, {1, 0, 1}, {1, 1, 0}, {1, 1, 0}};
    a.mx = c.met[0][kSt[comp][0]][2];
    a.my = c.met[1][kSt[comp][1]][2];
    a.mz = c.met[2][kSt[comp][2]][2];
    a.hy2hz2 = c.hy2hz2; a.hz2hx2 = c.hz2hx2; a.hx2hy2 = c.hx2hy2; a.h3 = c.hx2hy2hz2;
    a.Re = c.p.Re;
    a.ihx2 = 1.0 / (c.dXi[0] * c.dXi[0]); a.ihy2 = 1.0 / (c.dXi[1] * c.dXi[1]); a.ihz2 = 1.0 / (c.dXi[2] * c.dXi[2]);
    a.var = c.stretched ? 1 : 0;
    a.planar = c.planar ? 1 : 0;
    fa.rhs = a.rhs; fa.prog = a.prog; fa.full = a.full;
    fa.c1 = a.c1; fa.c2 = a.c2; fa.c3 = a.c3;
    fa.k1 = a.scalarForm ? (a.dt * a.coef) / a.X : a.dt / a.X;
    fa.invDn = 1.0 / a.Dn;
    fa.resMax = a.resMax;
}

// Split-FP64 solve buffers: N0 of components 0..3 and the D ping-pong, as
// float pairs of the largest padded component size.
static int cnp_ensure(Ctx &c) {
    if (c.cnp) return SARAS_OK;
    long n = 0;
    for (int fld : {SARAS_FIELD_VX, SARAS_FIELD_VY, SARAS_FIELD_VZ, SARAS_FIELD_T}) {
        const FieldInfo &f = c.info[fld];
        n = std::max(n, make_view<double>(nullptr, f.n[0], f.n[1], f.n[2]).size());
    }
    SARAS_CUDA_TRY(cudaMalloc(&c.cnp, sizeof(float) * 12 * (size_t)n));
    c.cnpCount = n;
    return SARAS_OK;
}

int compute_rhs(Ctx &c) {
    UC u = make_uc(c, SARAS_FIELD_VX);
    RhsArgs a;
    a.V = make_vel(c);
    a.P = cview(c, SARAS_FIELD_P);
    a.T = cview(c, SARAS_FIELD_T);
    a.u = u;
    a.visc = c.scalar ? c.nu : c.inverseRe;
    a.dt = c.dt;
    a.Fb = c.Fb;
    a.buoyancy = (c.scalar && c.p.forceType == 3) ? 1 : 0;
    double bytes = 0;
    prof_begin(c, PK_RHS, 0);
    RhsFast qf = make_rhs_fast(c, a.visc);
    bool fast = c.p.fastKernels != 0;
    Rhs3Args a3;   // fastKernels = 2: one k_rhs_df3 launch for the three components
    for (int q = 0; q < 3; ++q) {
        if (c.planar && q == 1) continue;   // hydro_d2.cc:222-240: Vx and Vz only
        a.H = mview(c, SARAS_FIELD_NSE_X + q);
        a.F = cview(c, SARAS_FIELD_VX + q);
        a.u = make_uc(c, SARAS_FIELD_VX + q);
        a.b = core_box(c.info[SARAS_FIELD_VX + q]);
        dim3 g, bl; box_launch_dims(a.b, g, bl);
        if (c.p.fastKernels == 2) {
            auto pr = [](double x) { fpair r; r.h = (float)x; r.l = (float)(x - (double)r.h); return r; };
            CnArgs ca;
            CnFast cfa;
            cn_setup(c, q, ca, cfa);
            const double kc[3] = {cfa.k1 * cfa.c1, cfa.k1 * cfa.c2, cfa.k1 * cfa.c3};
            Rhs3K qk;
            for (int d = 0; d < 3; ++d) {
                qk.kl[d] = pr((c.dt * qf.K2[d] + kc[d]) * cfa.invDn);
                qk.kn[d] = pr(c.dt * (qf.K1[d] / (q == d ? 1.0 : 4.0)) * cfa.invDn);   // Slices<q, d>::n
            }
            qk.kg = pr(c.dt * qf.G[q] * cfa.invDn);
            qk.kb = pr(c.dt * qf.Fb2 * cfa.invDn);
            int e = cnp_ensure(c);
            if (e) return e;
            float *n0h = c.cnp + (size_t)2 * q * c.cnpCount, *n0l = n0h + c.cnpCount;
            c.n0Fresh[q] = 1;
            {
                a3.n0h[q] = n0h;
                a3.n0l[q] = n0l;
                a3.q[q] = qk;
                bytes += 8.0 * (double)a.H.size();
                if (q < 2) continue;
                a3.f[0] = a.V.v[0].p; a3.f[1] = a.V.v[1].p; a3.f[2] = a.V.v[2].p;
                a3.f[3] = a.P.p;
                a3.T = a.T.p;
                for (int f = 0; f < 4; ++f) {
                    const View3<const double> &v = f < 3 ? a.V.v[f] : a.P;
                    for (int d = 0; d < 3; ++d) a3.n[f][d] = v.n[d];
                    a3.sx[f] = v.sx;
                    a3.sy[f] = v.sy;
                }
                for (int d = 0; d < 3; ++d) a3.nu[d] = std::max(std::max(a3.n[0][d], a3.n[1][d]), std::max(a3.n[2][d], a3.n[3][d]));
                a3.buoyancy = a.buoyancy;
                // rows of 32 m + 1 points: m tiles of 32 and one block column for the last point
                a3.edgeK = (a3.nu[2] > 32 && (a3.nu[2] - 1) % 32 == 0) ? a3.nu[2] - 1 : -1;
                dim3 gr(a3.edgeK >= 0 ? a3.edgeK / 32 + 1 : (a3.nu[2] + 31) / 32, (a3.nu[1] + 7) / 8,
                        (a3.nu[0] + kRhs3March - 1) / kRhs3March);
                if (rhs3_iso(a3)) k_rhs_df3<true><<<gr, dim3(32, 8, 1), 0, c.stream>>>(a3);
                else k_rhs_df3<false><<<gr, dim3(32, 8, 1), 0, c.stream>>>(a3);
                count_launch(c);
                break;
            }
        } else if (fast) {
            if (q == 0) k_rhs_fast<0><<<g, bl, 0, c.stream>>>(a, qf);
            if (q == 1) k_rhs_fast<1><<<g, bl, 0, c.stream>>>(a, qf);
            if (q == 2) k_rhs_fast<2><<<g, bl, 0, c.stream>>>(a, qf);
        } else {
            if (q == 0) k_rhs<0><<<g, bl, 0, c.stream>>>(a);
            if (q == 1) k_rhs<1><<<g, bl, 0, c.stream>>>(a);
            if (q == 2) k_rhs<2><<<g, bl, 0, c.stream>>>(a);
        }
        count_launch(c);
        bytes += 8.0 * (double)a.H.size();
    }
    // algorithmic bytes per point and component: F, two other velocity
    // components, P (+ T) in and H out; with fastKernels = 2 the four fields
    // (+ T) are read once for the three components and A (a float pair) is
    // written instead of H
    if (c.p.fastKernels == 2) prof_end(c, PK_RHS, 0, bytes * (a.buoyancy ? 8.0 : 7.0) / 3.0);
    else prof_end(c, PK_RHS, 0, bytes * (a.buoyancy ? 6.0 : 5.0));
    return check_launch(c, "rhs");
}

int compute_trhs(Ctx &c) {
    UC u = make_uc(c, SARAS_FIELD_T);
    RhsArgs a;
    a.V = make_vel(c);
    a.u = u;
    a.visc = c.kappa;
    a.dt = c.dt;
    a.H = mview(c, SARAS_FIELD_TRHS);
    a.F = cview(c, SARAS_FIELD_T);
    a.b = core_box(c.info[SARAS_FIELD_T]);
    dim3 g, bl; box_launch_dims(a.b, g, bl);
    k_trhs<<<g, bl, 0, c.stream>>>(a);
    count_launch(c);
    return check_launch(c, "trhs");
}

// fastKernels = 2: the delta-form split-FP64 Jacobi solve (k_cn_pack,
// k_cn_delta sweeps, k_cn_unpack), with the stopping rule and the sweep
// semantics of cn_solve: each sweep also reports the residual of its input,
// and the input of the first sweep whose input residual is below the
// tolerance is the answer.
static int cn_solve_delta(Ctx &c, int comp, int field, const CnFast &fa, double Dn, double bytes, int *iters, double *maxerr) {
    const FieldInfo &f = c.info[field];
    View3<double> V = mview(c, field);
    long n = V.size();
    int e = cnp_ensure(c);
    if (e) return e;
    long N = c.cnpCount;
    float *n0h = c.cnp + (size_t)2 * comp * N, *n0l = n0h + N;
    float *dA = c.cnp + (size_t)8 * N, *dAl = dA + N, *dB = dAl + N, *dBl = dB + N;
    CnDf fd = cn_df_consts(fa);
    if (!c.n0Fresh[comp]) {   // N0 not already written by the right-hand-side kernel
        dim3 g, bl; box_launch_dims(fa.full, g, bl);
        k_cn_pack<<<g, bl, 0, c.stream>>>(cview(c, field), fa.rhs, f.full, fa.full, fd, n0h, n0l);
        count_launch(c);
    }
    c.n0Fresh[comp] = 0;
    CnDelta d;
    d.C0 = V.p;
    d.n0h = n0h; d.n0l = n0l;
    d.sx = V.sx; d.sy = V.sy;
    d.prog = f.full;
    d.full = fa.full;
    d.f = fd;
    d.resMax = c.dscal;
    d.vout = nullptr;
    d.withResidual = 0;
    // The first iterate from D = 0 is A = N0 / Dn itself (on the bulk, written with
    // N0): its non-bulk points from their boundary-program sources, in place.
    d.dh = d.oh = n0h;
    d.dl = d.ol = n0l;
    k_cn_delta_shell<false, true><<<dim3(kShellBlocks, 6), 256, 0, c.stream>>>(d);
    count_launch(c);
    // The iterates: A (read only), then alternately P and Q.
    float *const bufs[3][2] = {{n0h, n0l}, {dA, dAl}, {dB, dBl}};
    int cur = 0, nxt = 1;
    auto advance = [&]() { int w = nxt; nxt = (w == 1) ? 2 : 1; cur = w; };
    dim3 gm((fa.full.ext[2] + 31) / 32, (fa.full.ext[1] + 7) / 8, (fa.full.ext[0] + kCnMarch - 1) / kCnMarch), bm(32, 8, 1);
    if (kCnColumns) {
        gm = dim3((unsigned)(((long)fa.full.ext[1] * fa.full.ext[2] + 255) / 256), (fa.full.ext[0] + kCnMarch - 1) / kCnMarch, 1);
        bm = dim3(256, 1, 1);
    }
    // vout: a final sweep, which writes C0 + D into vout (the field's scratch partner)
    // instead of D, the sum k_cn_unpack would form
    auto launch = [&](int withRes, double *vout) {
        d.dh = bufs[cur][0]; d.dl = bufs[cur][1]; d.oh = bufs[nxt][0]; d.ol = bufs[nxt][1];
        d.withResidual = withRes;
        d.vout = vout;
        prof_begin(c, PK_CN, 0);
        if (vout) {
            k_cn_delta<true><<<gm, bm, 0, c.stream>>>(d);
            k_cn_delta_shell<true, false><<<dim3(kShellBlocks, 6), 256, 0, c.stream>>>(d);
        } else {
            k_cn_delta<false><<<gm, bm, 0, c.stream>>>(d);
            k_cn_delta_shell<false, false><<<dim3(kShellBlocks, 6), 256, 0, c.stream>>>(d);
        }
        count_launch(c, 2);
        prof_end(c, PK_CN, 0, vout ? bytes * 4.0 / 3.0 : bytes);
    };
    auto read_res = [&](double &r) -> int {
        int s = check_launch(c, "cn");
        if (s) return s;
        SARAS_CUDA_TRY(cudaMemcpyAsync(c.hscal, c.dscal, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
        r = c.hscal[0] * Dn;
        return SARAS_OK;
    };
    // The Jacobi map contracts the max norm of successive corrections by
    // rho = 1 - 1/Dn (its off-diagonal weights over the diagonal; boundary
    // copies and reflections keep the weights' magnitudes), so the residual of
    // the iterate a sweep produced is at most rho * (that sweep's residual): when
    // that bound is below the tolerance, the sweep that would only confirm it is
    // skipped.
    const double rho = 1.0 - 1.0 / Dn;
    int sweeps = 1, failed = 0, status = SARAS_OK;   // sweep 1 (from D = 0) is A
    double res = 0;
    bool inField = false;   // the answer is already in the field (a final sweep was accepted)
    // Speculative final sweep: the sweeps the previous solve of this component
    // launched run without host round trips, the last of them as a final sweep.
    // If its residual bound meets the tolerance its output is the answer (no
    // unpack pass); if its own residual does, the previous iterate is, as in the
    // loop below; otherwise the loop resumes from that previous iterate.
    int slot = scratch_slot(field);
    int spec = slot >= 0 ? std::max(2, c.cnSweeps[comp]) : 0;
    if (spec > 0) {
        for (int q = 2; q < spec; ++q) {
            launch(0, nullptr);
            advance();
            sweeps += 1;
        }
        SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal, 0, sizeof(double), c.stream));
        launch(1, c.scratch[slot]);
        int s = read_res(res);
        if (s) return s;
        if (!std::isfinite(res)) {
            c.err = "Jacobi residual is not finite";
            status = SARAS_NOT_FINITE;
        } else if (res < c.p.cnTolerance && sweeps > 0) {
            c.cnSweeps[comp] = spec;   // cur (the previous iterate) is the answer
            spec = -1;
        } else if (res * rho * 1.01 < c.p.cnTolerance) {
            std::swap(c.f[field], c.scratch[slot]);
            c.cnSweeps[comp] = spec;
            sweeps = spec;
            res = res * rho * 1.01;
            inField = true;
            spec = -1;
        }
    }
    if (status == SARAS_OK && spec >= 0) {
        while (true) {
            SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal, 0, sizeof(double), c.stream));
            launch(1, nullptr);
            int s = read_res(res);
            if (s) return s;
            if (!std::isfinite(res)) { c.err = "Jacobi residual is not finite"; status = SARAS_NOT_FINITE; break; }
            if (res < c.p.cnTolerance) { c.cnSweeps[comp] = sweeps + 1; break; }   // cur is the answer
            double bound = res * rho * 1.01;
            if (bound < c.p.cnTolerance) {
                advance();
                sweeps += 1;
                res = bound;
                c.cnSweeps[comp] = sweeps;
                break;
            }
            failed += 1;
            if (failed > c.maxIterations) { status = SARAS_NOT_CONVERGED; break; }
            advance();
            sweeps += 1;
        }
    }
    // the field becomes C0 + D (also on failure, as the FP64 form leaves its last iterate)
    if (!inField) {
        k_cn_unpack<<<std::min<long>((n + 255) / 256, 152L * 16), 256, 0, c.stream>>>(V.p, bufs[cur][0], bufs[cur][1], n);
        count_launch(c);
        int s = check_launch(c, "cn unpack");
        if (s) return s;
    }
    if (iters) *iters = status == SARAS_NOT_CONVERGED ? failed : sweeps;
    if (maxerr) *maxerr = res;
    return status;
}

int cn_solve(Ctx &c, int comp, int *iters, double *maxerr) {
    if (comp < 0 || comp > 3) return SARAS_BAD_ARG;
    if (comp == 3 && !c.scalar) return SARAS_BAD_ARG;
    if (comp == 1 && c.planar) { c.err = "the 2D solver has no Vy equation"; return SARAS_BAD_ARG; }
    int field = comp == 3 ? SARAS_FIELD_T : SARAS_FIELD_VX + comp;
    const FieldInfo &f = c.info[field];
    CnArgs a;
    CnFast fa;
    cn_setup(c, comp, a, fa);
    dim3 g, bl; box_launch_dims(a.full, g, bl);
    int slot = scratch_slot(field);
    double bytes = 3.0 * 8.0 * (double)make_view<double>(nullptr, f.n[0], f.n[1], f.n[2]).size();
    bool fast = c.p.fastKernels != 0;
    const double resScale = fast ? a.Dn : 1.0;
    if (c.p.fastKernels == 2) return cn_solve_delta(c, comp, field, fa, a.Dn, bytes, iters, maxerr);
    auto launch = [&](int withRes) {
        if (fast) {
            fa.in = cview(c, field);
            fa.out = mview_ptr(c, field, c.scratch[slot]);
            fa.withResidual = withRes;
            k_cn_fast<<<g, bl, 0, c.stream>>>(fa);
        } else {
            a.in = cview(c, field);
            a.out = mview_ptr(c, field, c.scratch[slot]);
            a.withResidual = withRes;
            k_cn<<<g, bl, 0, c.stream>>>(a);
        }
    };
    // first sweep (no residual check precedes it)
    prof_begin(c, PK_CN, 0);
    launch(0);
    count_launch(c);
    prof_end(c, PK_CN, 0, bytes);
    std::swap(c.f[field], c.scratch[slot]);
    int sweeps = 1, failed = 0;
    double res = 0;
    while (true) {
        SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal, 0, sizeof(double), c.stream));
        prof_begin(c, PK_CN, 0);
        launch(1);
        count_launch(c);
        prof_end(c, PK_CN, 0, bytes);
        int s = check_launch(c, "cn");
        if (s) return s;
        SARAS_CUDA_TRY(cudaMemcpyAsync(c.hscal, c.dscal, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
        res = c.hscal[0] * resScale;
        if (!std::isfinite(res)) {
            c.err = "Jacobi residual is not finite";
            if (iters) *iters = sweeps;
            if (maxerr) *maxerr = res;
            return SARAS_NOT_FINITE;
        }
        if (res < c.p.cnTolerance) break;      // V_sweeps (the current field) is the answer
        failed += 1;
        if (failed > c.maxIterations) {
            if (iters) *iters = failed;
            if (maxerr) *maxerr = res;
            return SARAS_NOT_CONVERGED;
        }
        std::swap(c.f[field], c.scratch[slot]);
        sweeps += 1;
    }
    if (iters) *iters = sweeps;
    if (maxerr) *maxerr = res;
    return SARAS_OK;
}

// P += Pp over the padded array (hydro_d3.cc:357) and the velocity correction.
__global__ void k_add(double *dst, const double *src, long n, int zero_first) {
    long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    long stride = (long)gridDim.x * blockDim.x;
    for (; t < n; t += stride) dst[t] = (zero_first ? 0.0 : dst[t]) + src[t];
}

int project(Ctx &c, bool with_bc) {
    UC u = make_uc(c, SARAS_FIELD_P);
    long nP = make_view<double>(nullptr, c.info[SARAS_FIELD_P].n[0], c.info[SARAS_FIELD_P].n[1], c.info[SARAS_FIELD_P].n[2]).size();
    int blocks = (int)std::min<long>((nP + 255) / 256, 152L * 16);
    k_add<<<blocks, 256, 0, c.stream>>>(c.f[SARAS_FIELD_P], c.f[SARAS_FIELD_PP], nP, c.p.testPoisson ? 1 : 0);
    count_launch(c);
    prof_begin(c, PK_PROJECT, 0);
    double bytes = 0;
    for (int q = 0; q < 3; ++q) {
        if (c.planar && q == 1) continue;   // 2D: the y gradient is 0, Vy unchanged
        int field = SARAS_FIELD_VX + q;
        const FieldInfo &f = c.info[field];
        Box fb = full_box(f);
        dim3 g, bl; box_launch_dims(fb, g, bl);
        View3<double> out = mview_ptr(c, field, c.scratch[q]);
        View3<const double> in = cview(c, field), Pp = cview(c, SARAS_FIELD_PP);
        double fdt = u.gm[q] * u.ih[q] * c.dt;
        int wb = with_bc ? 1 : 0;
        if (c.p.fastKernels && with_bc) {
            const BcProgram &pg = f.full;
            dim3 gb((unsigned)(((long)(pg.bhi[2] - pg.blo[2] + 1) * (pg.bhi[1] - pg.blo[1] + 1) + 255) / 256),
                    (pg.bhi[0] - pg.blo[0] + 1 + kProjMarch - 1) / kProjMarch);
            dim3 gs(kShellBlocks, 6);
            if (q == 0) { k_project_bulk<0><<<gb, 256, 0, c.stream>>>(out, in, Pp, pg, fdt); k_project_shell<0><<<gs, 256, 0, c.stream>>>(out, in, Pp, pg, fb, fdt); }
            if (q == 1) { k_project_bulk<1><<<gb, 256, 0, c.stream>>>(out, in, Pp, pg, fdt); k_project_shell<1><<<gs, 256, 0, c.stream>>>(out, in, Pp, pg, fb, fdt); }
            if (q == 2) { k_project_bulk<2><<<gb, 256, 0, c.stream>>>(out, in, Pp, pg, fdt); k_project_shell<2><<<gs, 256, 0, c.stream>>>(out, in, Pp, pg, fb, fdt); }
            count_launch(c);
        } else if (c.p.fastKernels) {
            if (q == 0) k_project<0, true><<<g, bl, 0, c.stream>>>(out, in, Pp, f.full, fb, u, c.dt, wb, fdt);
            if (q == 1) k_project<1, true><<<g, bl, 0, c.stream>>>(out, in, Pp, f.full, fb, u, c.dt, wb, fdt);
            if (q == 2) k_project<2, true><<<g, bl, 0, c.stream>>>(out, in, Pp, f.full, fb, u, c.dt, wb, fdt);
        } else {
            if (q == 0) k_project<0, false><<<g, bl, 0, c.stream>>>(out, in, Pp, f.full, fb, u, c.dt, wb, fdt);
            if (q == 1) k_project<1, false><<<g, bl, 0, c.stream>>>(out, in, Pp, f.full, fb, u, c.dt, wb, fdt);
            if (q == 2) k_project<2, false><<<g, bl, 0, c.stream>>>(out, in, Pp, f.full, fb, u, c.dt, wb, fdt);
        }
        count_launch(c);
        std::swap(c.f[field], c.scratch[q]);
        bytes += 3.0 * 8.0 * (double)out.size();
    }
    prof_end(c, PK_PROJECT, 0, bytes);
    return check_launch(c, "project");
}

int reduce_sum_partials(Ctx &c, int nparts, double *host_out) {
    k_final_reduce<<<1, 256, 0, c.stream>>>(c.red, nparts, 0, c.dscal + 8);
    count_launch(c);
    SARAS_CUDA_TRY(cudaMemcpyAsync(c.hscal + 8, c.dscal + 8, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    *host_out = c.hscal[8];
    return SARAS_OK;
}

int diagnostics(Ctx &c, double *energy, double *maxdiv, double *nusselt) {
    UC u = make_uc(c, SARAS_FIELD_P);
    int nb = 152 * 4;
    if (nb > c.redCap) nb = c.redCap;
    double dv = (c.dXi[0] / c.m1[0]) * (c.dXi[1] / c.m1[1]) * (c.dXi[2] / c.m1[2]);
    k_diag<<<nb, 256, 0, c.stream>>>(make_vel(c), cview(c, SARAS_FIELD_T), c.scalar ? 1 : 0, c.Ns[0], c.Ns[1], c.Ns[2],
                                     c.Nc[0], c.Nc[1], c.Nc[2], u, dv, c.red, c.red + c.redCap, c.red + 2 * c.redCap);
    count_launch(c);
    k_final_reduce<<<1, 256, 0, c.stream>>>(c.red, nb, 0, c.dscal + 10);
    k_final_reduce<<<1, 256, 0, c.stream>>>(c.red + c.redCap, nb, 0, c.dscal + 11);
    k_final_reduce<<<1, 256, 0, c.stream>>>(c.red + 2 * c.redCap, nb, 1, c.dscal + 12);
    count_launch(c, 3);
    SARAS_CUDA_TRY(cudaMemcpyAsync(c.hscal + 10, c.dscal + 10, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    int s = check_launch(c, "diagnostics");
    if (s) return s;
    if (energy) *energy = c.hscal[10] / c.totalVol;
    if (maxdiv) *maxdiv = c.hscal[12];
    if (nusselt) *nusselt = c.scalar ? 1.0 + (c.hscal[11] / c.totalVol) / c.kappa : 0.0;
    return c.hscal[12] > 1.0e5 ? SARAS_DIVERGENCE_LIMIT : SARAS_OK;
}

// max |F| over a whole padded array (field::fieldMax, field.cc:602-617): exact in any order.
__global__ void k_field_maxabs(const double *a, long n, double *out) {
    double m = 0;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        double v = fabs(a[t]);
        if (v != v) v = INFINITY;
        m = fmax(m, v);
    }
    block_max_to(m, out);
}

// vfield::computeTStp (vfield.cc:267-284): dt = courantNumber (dXi / Umax +
// dEt / Vmax + dZt / Wmax) with U/V/Wmax = fieldMax of Vx/Vy/Vz, in the
// reference's operation order (a zero maximum gives an infinite term, which
// solvePDE's cap at "Time-Step" then replaces, hydro_d3.cc:196-203).
int compute_tstp(Ctx &c, double *dt) {
    SARAS_CUDA_TRY(cudaMemsetAsync(c.dscal + 48, 0, 3 * sizeof(double), c.stream));
    for (int q = 0; q < 3; ++q) {
        long n = mview(c, SARAS_FIELD_VX + q).size();
        int nb = (int)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 4));
        k_field_maxabs<<<nb, 256, 0, c.stream>>>(c.f[SARAS_FIELD_VX + q], n, c.dscal + 48 + q);
    }
    count_launch(c, 3);
    SARAS_CUDA_TRY(cudaMemcpyAsync(c.hscal + 48, c.dscal + 48, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    int s = check_launch(c, "computeTStp");
    if (s) return s;
    const double Umax = c.hscal[48], Vmax = c.planar ? 1.0 : c.hscal[49], Wmax = c.hscal[50];
    const double dely = c.planar ? 0.0 : c.dXi[1];   // vfield.cc:273-279
    *dt = c.p.courantNumber * (c.dXi[0] / Umax + dely / Vmax + c.dXi[2] / Wmax);
    return SARAS_OK;
}

// probes::getData (probes.cc:174-189): the value of each field at each probe
// point (logical indices of the field's padded array); out[p * nf + f].
struct ProbeFields {
    const double *f[SARAS_NUM_FIELDS];
    long sx[SARAS_NUM_FIELDS], sy[SARAS_NUM_FIELDS];
};
__global__ void k_probe(const int *ijk, int n, ProbeFields pf, int nf, double *out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * nf) return;
    int p = t / nf, f = t - p * nf;
    const int i = ijk[3 * p], j = ijk[3 * p + 1], k = ijk[3 * p + 2];
    out[t] = pf.f[f][(long)(i + 1) * pf.sx[f] + (long)(j + 1) * pf.sy[f] + (k + 1)];
}

int probe(Ctx &c, int n, const int *ijk, int nf, const int *fields, double *out) {
    if (n < 0 || nf < 0 || nf > SARAS_NUM_FIELDS || (n > 0 && (!ijk || !out)) || (nf > 0 && !fields)) return SARAS_BAD_ARG;
    if (n == 0 || nf == 0) return SARAS_OK;
    ProbeFields pf;
    for (int q = 0; q < nf; ++q) {
        if (fields[q] < 0 || fields[q] >= SARAS_NUM_FIELDS) return SARAS_BAD_ARG;
        View3<double> v = mview(c, fields[q]);
        pf.f[q] = v.p; pf.sx[q] = v.sx; pf.sy[q] = v.sy;
        for (int p = 0; p < n; ++p)
            for (int d = 0; d < 3; ++d)
                if (ijk[3 * p + d] < -1 || ijk[3 * p + d] > v.n[d]) {
                    c.err = "probe index outside the padded field";
                    return SARAS_BAD_ARG;
                }
    }
    const size_t need = sizeof(int) * 3 * (size_t)n + sizeof(double) * (size_t)n * nf + 256;
    if (need > c.probeBytes) {
        cudaFree(c.probeBuf);
        c.probeBuf = nullptr;
        c.probeBytes = 0;
        SARAS_CUDA_TRY(cudaMalloc(&c.probeBuf, need));
        c.probeBytes = need;
    }
    int *dijk = reinterpret_cast<int *>(c.probeBuf);
    double *dout = reinterpret_cast<double *>(static_cast<char *>(c.probeBuf) + ((sizeof(int) * 3 * (size_t)n + 255) / 256) * 256);
    SARAS_CUDA_TRY(cudaMemcpyAsync(dijk, ijk, sizeof(int) * 3 * (size_t)n, cudaMemcpyHostToDevice, c.stream));
    k_probe<<<(n * nf + 255) / 256, 256, 0, c.stream>>>(dijk, n, pf, nf, dout);
    count_launch(c);
    SARAS_CUDA_TRY(cudaMemcpyAsync(out, dout, sizeof(double) * (size_t)n * nf, cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return check_launch(c, "probes");
}

// hydro_d3::testPeriodic (hydro_d3.cc:536-679): fill Vx, Vy (and the expected
// arrays) on the host, impose the velocity BCs on the device, compare.
int hydro_test_periodic(Ctx &c, double *err) {
    const double PI = M_PI;
    auto coordS = [&](int d, int i) { return c.L[d] * (double(i) * c.dXi[d]); };
    auto coordC = [&](int d, int i) { return c.L[d] * (double(i) * c.dXi[d] + double(i + 1) * c.dXi[d]) / 2.0; };
    double worst = 0.0;
    for (int q = 0; q < 2; ++q) {
        int field = SARAS_FIELD_VX + q;
        const FieldInfo &f = c.info[field];
        int nx = f.n[0], ny = f.n[1], nz = f.n[2];
        View3<double> hv = make_view<double>(nullptr, nx, ny, nz);
        std::vector<double> V(hv.size()), E(hv.size());
        auto fn = [&](double x, double y, double z) {
            return q == 0 ? std::sin(2.0 * PI * x / c.L[0]) * std::cos(2.0 * PI * y / c.L[1]) * std::cos(2.0 * PI * z / c.L[2])
                          : -std::cos(2.0 * PI * x / c.L[0]) * std::sin(2.0 * PI * y / c.L[1]) * std::cos(2.0 * PI * z / c.L[2]);
        };
        auto X = [&](int d, int i) { return f.stag[d] ? coordS(d, i) : coordC(d, i); };
        for (int i = -1; i <= nx; ++i) for (int j = -1; j <= ny; ++j) for (int k = -1; k <= nz; ++k)
            V[hv.off(i, j, k)] = E[hv.off(i, j, k)] = fn(X(0, i), X(1, j), X(2, k));
        int n3[3] = {nx, ny, nz};
        for (int d = 0; d < 3; ++d) {
            double lo = X(d, 0) - (X(d, 1) - X(d, 0));
            double hi = X(d, n3[d] - 1) + (X(d, n3[d] - 1) - X(d, n3[d] - 2));
            int a1 = (d + 1) % 3, a2 = (d + 2) % 3;
            for (int s = 0; s < n3[a1]; ++s) for (int t = 0; t < n3[a2]; ++t) {
                int pl[3], ph[3];
                pl[d] = -1; ph[d] = n3[d]; pl[a1] = ph[a1] = s; pl[a2] = ph[a2] = t;
                double cl[3], ch[3];
                for (int e = 0; e < 3; ++e) { cl[e] = X(e, pl[e]); ch[e] = X(e, ph[e]); }
                cl[d] = lo; ch[d] = hi;
                E[hv.off(pl[0], pl[1], pl[2])] = fn(cl[0], cl[1], cl[2]);
                E[hv.off(ph[0], ph[1], ph[2])] = fn(ch[0], ch[1], ch[2]);
            }
        }
        SARAS_CUDA_TRY(cudaMemcpyAsync(c.f[field], V.data(), V.size() * 8, cudaMemcpyHostToDevice, c.stream));
        int s = apply_bc(c, field);
        if (s) return s;
        SARAS_CUDA_TRY(cudaMemcpyAsync(V.data(), c.f[field], V.size() * 8, cudaMemcpyDeviceToHost, c.stream));
        SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
        for (size_t n = 0; n < V.size(); ++n) worst = std::max(worst, std::fabs(V[n] - E[n]));
    }
    *err = worst;
    return SARAS_OK;
}

// hydro_d3::timeAdvance (hydro_d3.cc:254-368) / scalar_d3::timeAdvance (scalar_d3.cc:243-370)
int time_advance(Ctx &c, saras_step_stats *st) {
    saras_step_stats local;
    std::memset(&local, 0, sizeof(local));
    int s = compute_rhs(c);
    if (s) { for (int &q : c.n0Fresh) q = 0; return s; }
    for (int q = 0; q < 3; ++q) {
        if (c.planar && q == 1) continue;   // hydro_d2.cc:242-244: solveVx, solveVz
        int it = 0; double e = 0;
        s = cn_solve(c, q, &it, &e);
        local.cn_iters[q] = it;
        if (s) { for (int &r : c.n0Fresh) r = 0; local.status = s; if (st) *st = local; return s; }
    }
    s = vfield_divergence(c, nullptr, true);
    if (s) return s;
    int cyc = 0; double res = 0;
    s = mg_solve(c, &cyc, &res, &local);
    local.vcycles = cyc;
    local.mg_residual = res;
    if (s) { local.status = s; if (st) *st = local; return s; }
    s = sync_field(c, SARAS_FIELD_PP);
    if (s) return s;
    s = project(c, !c.scalar);
    if (s) return s;
    if (c.scalar) {
        s = compute_trhs(c);
        if (s) return s;
        int it = 0; double e = 0;
        s = cn_solve(c, 3, &it, &e);
        local.cn_iters[3] = it;
        if (s) { local.status = s; if (st) *st = local; return s; }
        for (int q = 0; q < 3; ++q) {
            if (c.planar && q == 1) continue;   // scalar_d2.cc:309-311: imposeUBCs, imposeWBCs, imposeTBCs
            s = apply_bc(c, SARAS_FIELD_VX + q);
            if (s) return s;
        }
        s = apply_bc(c, SARAS_FIELD_T);
        if (s) return s;
    }
    c.last = local;
    if (st) *st = local;
    return SARAS_OK;
}

}  // namespace saras

// ------------------------------------------------------------------ allocation-free Jacobi solve
// Some callers cannot allocate device memory at the point where they need a
// solve: a host application that hands the solver a fixed memory budget up
// front, a caller running under a custom pool allocator that forbids further
// cudaMalloc/cudaFree traffic once its simulation loop has started, or code
// that must not change the device's allocation state between two checkpoints.
// saras_cn_solve_noalloc serves them: the caller passes the velocity (or
// temperature) array and the right-hand side in device memory, and the second
// iterate plus the residual slot live in the fixed array below instead of in
// memory from cudaMalloc.  The array is reserved on every GPU that loads the
// library, for the life of the process, whether or not this entry point is
// used.
namespace saras {

constexpr long kNoAllocMaxPoints = 4L << 20;   // 4 Mi doubles (32 MiB): padded field arrays up to this size
static __device__ __align__(256) double g_cn_scratch[kNoAllocMaxPoints + 32];
// Device address of g_cn_scratch, per device ordinal.  Atomic: two host
// threads making their first call on a device at the same time both look the
// address up and store the same value, without a data race on the slot.
static std::atomic<double *> g_cn_scratch_dev[64];

// The wall objects of walls_for(), written into a fixed array (no host heap use).
static int walls_fixed(const saras_params &p, int field, Wall *w) {
    int n = 0;
    auto add = [&](WallKind k, int wall, double v) { w[n++] = Wall{k, wall, v}; };
    if (field == SARAS_FIELD_VX) {
        if (!p.xPer) { if (p.probType == 3) { add(W_DIR_FC, 0, 1.0); add(W_NEU, 1, 0.0); } else { add(W_DIR_FC, 0, 0.0); add(W_DIR_FC, 1, 0.0); } }
        if (!p.yPer) { add(W_DIR_CC, 2, 0.0); add(W_DIR_CC, 3, 0.0); }
        if (p.zPer) { add(W_PER_CC, 5, 0); add(W_PER_CC, 4, 0); }
        else if (p.probType == 1) { add(W_DIR_CC, 5, 1.0); add(W_DIR_CC, 4, 0.0); }
        else { add(W_DIR_CC, 5, 0.0); add(W_DIR_CC, 4, 0.0); }
    } else if (field == SARAS_FIELD_VY) {
        if (!p.xPer) { if (p.probType == 3) { add(W_DIR_CC, 0, 0.0); add(W_NEU, 1, 0.0); } else { add(W_DIR_CC, 0, 0.0); add(W_DIR_CC, 1, 0.0); } }
        if (!p.yPer) { add(W_DIR_FC, 2, 0.0); add(W_DIR_FC, 3, 0.0); }
        if (p.zPer) { add(W_PER_CC, 5, 0); add(W_PER_CC, 4, 0); }
        else { add(W_DIR_CC, 5, 0.0); add(W_DIR_CC, 4, 0.0); }
    } else if (field == SARAS_FIELD_VZ) {
        if (!p.xPer) { if (p.probType == 3) { add(W_DIR_CC, 0, 0.0); add(W_NEU, 1, 0.0); } else { add(W_DIR_CC, 0, 0.0); add(W_DIR_CC, 1, 0.0); } }
        if (!p.yPer) { add(W_DIR_CC, 2, 0.0); add(W_DIR_CC, 3, 0.0); }
        if (p.zPer) { add(W_PER_FC, 5, 0); add(W_PER_FC, 4, 0); }
        else { add(W_DIR_FC, 5, 0.0); add(W_DIR_FC, 4, 0.0); }
    } else {
        if (!p.xPer) {
            if (p.probType == 5 || p.probType == 6 || p.probType == 8) { add(W_NEU, 0, 0.0); add(W_NEU, 1, 0.0); }
            else if (p.probType == 7) { add(W_DIR_CC, 0, 1.0); add(W_DIR_CC, 1, 0.0); }
        }
        if (!p.yPer) { add(W_NEU, 2, 0.0); add(W_NEU, 3, 0.0); }
        if (p.zPer) { add(W_PER_CC, 5, 0); add(W_PER_CC, 4, 0); }
        else if (p.probType == 5 || p.probType == 8) { add(W_DIR_CC, 5, 0.0); add(W_DIR_CC, 4, 1.0); }
        else if (p.probType == 6) { add(W_DIR_CC, 5, 1.0); add(W_DIR_CC, 4, 0.0); }
    }
    return n;
}

}  // namespace saras

// The same Jacobi iteration as saras_cn_solve (same kernels, same stopping
// rule and iteration cap) for fastKernels 0 and 1, on caller-owned device
// arrays v (in: current iterate with its boundary values, out: solution) and
// rhs; with fastKernels = 2 it runs the fastKernels = 1 iteration (the same
// system and stopping rule in FP64 fused multiply-adds, where saras_cn_solve
// runs the split-FP64 delta form).  Nothing is allocated.  The first call on a device looks up the device address of the
// scratch array; make that first call before any stream capture.  Every call
// shares the one array, so calls that overlap on the GPU (other streams,
// other host threads) race: order them on one stream or serialise them.
extern "C" int saras_cn_solve_noalloc(const saras_params *p, int component, double *v, const double *rhs, void *stream,
                                      int *iters, double *max_error) {
    using namespace saras;
    if (!p || !v || !rhs) return SARAS_BAD_ARG;
    bool scalar = p->probType >= 5;
    if (component < 0 || component > 3 || (component == 3 && !scalar)) return SARAS_BAD_ARG;
    if (p->xGrid || p->yGrid || p->zGrid || p->xInd < 2 || p->yInd < 2 || p->zInd < 2 || p->xInd > 11 || p->yInd > 11 || p->zInd > 11)
        return SARAS_BAD_CONFIG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); set_error("no CUDA device"); return SARAS_NO_DEVICE; }
    if (dev < 0 || dev >= 64) { set_error("device ordinal beyond 63"); return SARAS_BAD_ARG; }
    double *scratch = g_cn_scratch_dev[dev].load(std::memory_order_acquire);
    if (!scratch) {
        cudaError_t e = cudaGetSymbolAddress((void **)&scratch, g_cn_scratch);
        if (e != cudaSuccess || !scratch) {
            set_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            return SARAS_CUDA_ERROR;
        }
        g_cn_scratch_dev[dev].store(scratch, std::memory_order_release);
    }
    double *resSlot = scratch + kNoAllocMaxPoints;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

    // grid constants (grid.cc:84-86, 405-421; hydro.cc:223-241)
    int ind[3] = {p->xInd, p->yInd, p->zInd};
    double L[3] = {p->Lx, p->Ly, p->Lz};
    double dXi[3], m2[3];
    int Ns[3], Nc[3];
    for (int d = 0; d < 3; ++d) {
        Ns[d] = int(std::pow(2, ind[d])) + 1;
        Nc[d] = Ns[d] - 1;
        dXi[d] = 1.0 / double(Ns[d] - 1);
        m2[d] = std::pow(1.0 / L[d], 2.0);
    }
    double hz2hx2 = std::pow(dXi[2], 2.0) * std::pow(dXi[0], 2.0);
    double hx2hy2 = std::pow(dXi[0], 2.0) * std::pow(dXi[1], 2.0);
    double hy2hz2 = std::pow(dXi[1], 2.0) * std::pow(dXi[2], 2.0);
    double hx2hy2hz2 = std::pow(dXi[0], 2.0) * std::pow(dXi[1], 2.0) * std::pow(dXi[2], 2.0);
    int maxIterations = Nc[0] * Nc[1] * Nc[2];

    // field layout, bulk box and boundary program (field.cc:66-290, hydro.cc:287-461)
    int field = component == 3 ? SARAS_FIELD_T : SARAS_FIELD_VX + component;
    bool stg[3] = {field != SARAS_FIELD_VX, field != SARAS_FIELD_VY, field != SARAS_FIELD_VZ};
    bool per[3] = {p->xPer != 0, p->yPer != 0, p->zPer != 0};
    FieldInfo f;
    for (int d = 0; d < 3; ++d) {
        f.stag[d] = stg[d];
        f.n[d] = stg[d] ? Ns[d] : Nc[d];
        f.blo[d] = 0; f.bhi[d] = f.n[d] - 1;
        if (stg[d] && !per[d]) { f.blo[d] += 1; f.bhi[d] -= 1; }
    }
    long points = (long)(f.n[0] + 2) * (f.n[1] + 2) * (f.n[2] + 2);
    if (points > kNoAllocMaxPoints) {
        set_error("saras_cn_solve_noalloc: field of " + std::to_string(points) + " points exceeds the fixed scratch of " +
                  std::to_string(kNoAllocMaxPoints) + " points; use saras_cn_solve");
        return SARAS_TOO_LARGE;
    }
    f.full.nops = 0;
    add_sync_ops(f.full, f, per[0], per[1], false);   // 3D only (yInd >= 2 checked above)
    Wall walls[6];
    int nw = walls_fixed(*p, field, walls);
    for (int q = 0; q < nw; ++q) add_wall_op(f.full, f, walls[q]);
    for (int d = 0; d < 3; ++d) { f.full.blo[d] = f.blo[d]; f.full.bhi[d] = f.bhi[d]; }

    // coefficients, as in cn_solve
    double nu = 0, kappa = 0;
    if (scalar) {
        if (p->rbcType == 1) { nu = p->Pr; kappa = 1.0; }
        else if (p->rbcType == 3) { nu = 1.0; kappa = 1.0 / p->Pr; }
        else { nu = std::sqrt(p->Pr / p->Ra); kappa = 1.0 / std::sqrt(p->Pr * p->Ra); }
    }
    CnArgs a;
    a.var = 0;   // uniform 3D meshes only (checked above)
    a.planar = 0;
    a.mx = a.my = a.mz = nullptr;
    {
        View3<double> w = make_view<double>(const_cast<double *>(rhs), f.n[0], f.n[1], f.n[2]);
        a.rhs.p = w.p; a.rhs.n[0] = w.n[0]; a.rhs.n[1] = w.n[1]; a.rhs.n[2] = w.n[2]; a.rhs.sx = w.sx; a.rhs.sy = w.sy;
    }
    a.prog = f.full;
    Box fb; for (int d = 0; d < 3; ++d) { fb.lo[d] = -1; fb.ext[d] = f.n[d] + 2; }
    a.full = fb;
    a.c1 = hy2hz2 * m2[0]; a.c2 = hz2hx2 * m2[1]; a.c3 = hx2hy2 * m2[2];
    double B = (hy2hz2 * m2[0] + hz2hx2 * m2[1]) + hx2hy2 * m2[2];
    a.dt = p->tStp;
    if (!scalar) {
        a.scalarForm = 0; a.coef = 0;
        a.X = hx2hy2hz2 * 2.0 * p->Re;
        a.Dn = 1.0 + p->tStp * B / (p->Re * hx2hy2hz2);
        a.iX = 1.0 / a.X;
        a.iDn = 1.0 / a.Dn;
        a.resCoef = 1.0 / p->Re;
    } else {
        double coef = component == 3 ? kappa : nu;
        a.scalarForm = 1; a.coef = coef;
        a.X = hx2hy2hz2 * 2.0;
        a.Dn = 1.0 + p->tStp * coef * B / hx2hy2hz2;
        a.iX = 1.0 / a.X;
        a.iDn = 1.0 / a.Dn;
        a.resCoef = coef;
    }
    a.lx = m2[0] * (1.0 / (dXi[0] * dXi[0]));
    a.ly = m2[1] * (1.0 / (dXi[1] * dXi[1]));
    a.lz = m2[2] * (1.0 / (dXi[2] * dXi[2]));
    a.resMax = resSlot;
    dim3 g, bl; box_launch_dims(fb, g, bl);

    // the fused multiply-add form when the parameters ask for it, as cn_solve does
    CnFast fa;
    bool fast = p->fastKernels != 0;
    if (fast) {
        fa.rhs = a.rhs; fa.prog = a.prog; fa.full = a.full;
        fa.c1 = a.c1; fa.c2 = a.c2; fa.c3 = a.c3;
        fa.k1 = a.scalarForm ? (a.dt * a.coef) / a.X : a.dt / a.X;
        fa.invDn = 1.0 / a.Dn;
        fa.resMax = a.resMax;
    }
    const double resScale = fast ? a.Dn : 1.0;
    double *cur = v, *nxt = scratch;
    auto view_of = [&](double *ptr) { return make_view<double>(ptr, f.n[0], f.n[1], f.n[2]); };
    auto launch = [&](int withRes) {
        View3<double> in = view_of(cur), out = view_of(nxt);
        View3<const double> cin;
        cin.p = in.p; cin.n[0] = in.n[0]; cin.n[1] = in.n[1]; cin.n[2] = in.n[2]; cin.sx = in.sx; cin.sy = in.sy;
        if (fast) {
            fa.in = cin; fa.out = out; fa.withResidual = withRes;
            // fastKernels 1 and 2 both run this fused multiply-add form: the
            // split-FP64 form of fastKernels = 2 keeps N0 and the correction
            // as float pairs, 12 more floats a point than the fixed array holds
            k_cn_fast<<<g, bl, 0, st>>>(fa);
        } else {
            a.in = cin; a.out = out; a.withResidual = withRes;
            k_cn<<<g, bl, 0, st>>>(a);
        }
        return cudaGetLastError();
    };
    cudaError_t e = launch(0);
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return SARAS_CUDA_ERROR; }
    std::swap(cur, nxt);
    int sweeps = 1, failed = 0;
    double res = 0.0;
    int status = SARAS_OK;
    while (true) {
        if ((e = cudaMemsetAsync(resSlot, 0, sizeof(double), st)) != cudaSuccess) break;
        if ((e = launch(1)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(&res, resSlot, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
        res *= resScale;
        if (!std::isfinite(res)) { set_error("Jacobi residual is not finite"); status = SARAS_NOT_FINITE; break; }
        if (res < p->cnTolerance) break;
        failed += 1;
        if (failed > maxIterations) { status = SARAS_NOT_CONVERGED; break; }
        std::swap(cur, nxt);
        sweeps += 1;
    }
    if (e != cudaSuccess) { set_error(cudaGetErrorString(e)); return SARAS_CUDA_ERROR; }
    // the answer is `cur`; bring it into the caller's array if it sits in the scratch
    if (cur != v) {
        if ((e = cudaMemcpyAsync(v, cur, sizeof(double) * points, cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            set_error(cudaGetErrorString(e));
            return SARAS_CUDA_ERROR;
        }
    }
    if (iters) *iters = status == SARAS_NOT_CONVERGED ? failed : sweeps;
    if (max_error) *max_error = res;
    return status;
}
