// saras_oracle.cc -- CPU restatement of the SARAS per-time-step hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300
// kernels: tests, the smoke check and the CPU-baseline leg of the benchmark
// load it; the product library never does.  It restates, loop by loop, the
// reference's own CPU algorithm at np = 1 (every MPI call replaced by its
// single-rank meaning) and is compiled with strict IEEE arithmetic
// (-O2 -ffp-contract=off), so that each floating-point expression is evaluated
// in the reference's order.  Every function cites the reference file:line it
// follows (paths inside the roshansamuel/saras repository).
//
// Pinning: Blitz++ (third-party, unpinned git HEAD, not vendored in the
// reference) owns the stencil operators central12n / central22n, the array
// reductions and the evaluation domain of stencil expressions.  They are
// restated from Blitz++'s published definitions:
//   central12n(A,d) = (A[+1] - A[-1]) * 0.5,
//   central22n(A,d) = A[-1] - 2*A[0] + A[+1]   (evaluated left to right),
// evaluated at every index of the destination range, i.e. the result at i uses
// A[i-1], A[i], A[i+1].  The reference's own tests pin these only to O(h)
// (nlin_test.cc:77, field_test.cc:51-76); the known-answer tests of
// poisson_d3.cc:689-857 and hydro_d3.cc:536-679 pin the transfer, ghost and
// prolongation operators exactly.  See tests/test_oracle_kats.py.

#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>
#include <utility>

#include "../include/saras_gb300.h"

namespace {

// ------------------------------------------------------------------ arrays
// Blitz-like 3D array with arbitrary lower bounds, C order (k fastest).
struct A3 {
    int lb[3] = {0, 0, 0}, ub[3] = {-1, -1, -1};
    long n[3] = {0, 0, 0};
    long sx = 0, sy = 0;
    std::vector<double> v;
    void resize(int l0, int l1, int l2, int u0, int u1, int u2) {
        lb[0] = l0; lb[1] = l1; lb[2] = l2; ub[0] = u0; ub[1] = u1; ub[2] = u2;
        for (int d = 0; d < 3; ++d) n[d] = ub[d] - lb[d] + 1;
        sy = n[2]; sx = n[1] * n[2];
        v.assign((size_t)(n[0] * n[1] * n[2]), 0.0);
    }
    inline double &operator()(int i, int j, int k) {
        return v[(size_t)((i - lb[0]) * sx + (j - lb[1]) * sy + (k - lb[2]))];
    }
    inline double operator()(int i, int j, int k) const {
        return v[(size_t)((i - lb[0]) * sx + (j - lb[1]) * sy + (k - lb[2]))];
    }
    void fill(double a) { std::fill(v.begin(), v.end(), a); }
    size_t size() const { return v.size(); }
};

struct A1 {  // 1D array with lower bound
    int lb = 0;
    std::vector<double> v;
    void resize(int l, int u) { lb = l; v.assign((size_t)(u - l + 1), 0.0); }
    inline double &operator()(int i) { return v[(size_t)(i - lb)]; }
    inline double operator()(int i) const { return v[(size_t)(i - lb)]; }
};

// Sum of a sequence in fixed 4096-element chunks: each chunk is summed in
// index order, then the chunk sums are summed in chunk order.  The GPU
// reduction of the same sums follows exactly this order, so both sides agree
// bit for bit (the reference's one-pass Blitz sum differs from it by rounding).
static const long kChunk = 4096;
template <class Get>
static double chunked_sum(long n, Get get) {
    double total = 0.0;
    for (long c0 = 0; c0 < n; c0 += kChunk) {
        double s = 0.0;
        long c1 = std::min(n, c0 + kChunk);
        for (long t = c0; t < c1; ++t) s += get(t);
        total += s;
    }
    return total;
}

// Blitz++ stencil operators (see header comment).
static inline double central12n(double fm, double fp) { return (fp - fm) * 0.5; }
static inline double central22n(double fm, double f0, double fp) { return fm - 2.0 * f0 + fp; }

// ------------------------------------------------------------------ grid
// grid.cc:59-136, 176-255, 333-422 at np = 1 with uniform ("UUU") meshes.
struct Grid {
    int sizeIndex[3];
    int globalSize[3];
    double dXi, dEt, dZt;
    double xLen, yLen, zLen;
    int staggrCoreSize[3], collocCoreSize[3];
    A1 xi, et, zt;
    A1 xStaggr, yStaggr, zStaggr, xColloc, yColloc, zColloc;
    A1 xi_xColloc, xixxColloc, xix2Colloc, et_yColloc, etyyColloc, ety2Colloc, zt_zColloc, ztzzColloc, ztz2Colloc;
    A1 xi_xStaggr, xixxStaggr, xix2Staggr, et_yStaggr, etyyStaggr, ety2Staggr, zt_zStaggr, ztzzStaggr, ztz2Staggr;
    // the 2D (PLANAR) solver: "Y Index" 0 gives one y point, dEt = yLen = 1
    // (grid.cc:88-92) and one collocated y point (grid.cc:232-234)
    bool planar = false;

    void build(const saras_params &p) {
        planar = p.yInd == 0;
        sizeIndex[0] = p.xInd; sizeIndex[1] = p.yInd; sizeIndex[2] = p.zInd;
        for (int d = 0; d < 3; ++d) globalSize[d] = (sizeIndex[d] == 0) ? 1 : (int(std::pow(2, sizeIndex[d])) + 1);
        xLen = p.Lx; yLen = p.Ly; zLen = p.Lz;
        dXi = 1.0 / double(globalSize[0] - 1);
        dEt = 1.0 / double(globalSize[1] - 1);
        dZt = 1.0 / double(globalSize[2] - 1);
        if (planar) { yLen = 1.0; dEt = 1.0; }
        for (int d = 0; d < 3; ++d) {
            staggrCoreSize[d] = globalSize[d];           // grid.cc:182-188 at npX = npY = 1
            collocCoreSize[d] = staggrCoreSize[d] - 1;   // grid.cc:230
        }
        if (planar) collocCoreSize[1] = 1;
        // grid.cc:333-352 (global transformed grid = local at np = 1)
        xi.resize(-1, globalSize[0]); et.resize(-1, globalSize[1]); zt.resize(-1, globalSize[2]);
        for (int i = -1; i < globalSize[0] + 1; i++) xi(i) = double(i) * dXi;
        for (int i = -1; i < globalSize[1] + 1; i++) et(i) = double(i) * dEt;
        for (int i = -1; i < globalSize[2] + 1; i++) zt(i) = double(i) * dZt;
        int sx = staggrCoreSize[0], sy = staggrCoreSize[1], sz = staggrCoreSize[2];
        int cx = collocCoreSize[0], cy = collocCoreSize[1], cz = collocCoreSize[2];
        A1 *stg[3][3] = {{&xi_xStaggr, &xixxStaggr, &xix2Staggr}, {&et_yStaggr, &etyyStaggr, &ety2Staggr}, {&zt_zStaggr, &ztzzStaggr, &ztz2Staggr}};
        A1 *col[3][3] = {{&xi_xColloc, &xixxColloc, &xix2Colloc}, {&et_yColloc, &etyyColloc, &ety2Colloc}, {&zt_zColloc, &ztzzColloc, &ztz2Colloc}};
        int sc[3] = {sx, sy, sz}, cc[3] = {cx, cy, cz};
        double L[3] = {xLen, yLen, zLen};
        for (int d = 0; d < 3; ++d) {
            for (int m = 0; m < 3; ++m) { stg[d][m]->resize(-1, sc[d]); col[d][m]->resize(-1, cc[d]); }
            // grid.cc:314-320 defaults, then createUniformGrid grid.cc:405-421
            double inv = 1.0 / L[d];
            double inv2 = std::pow(inv, 2.0);
            for (auto &x : stg[d][0]->v) x = inv;
            for (auto &x : stg[d][1]->v) x = 0.0;
            for (auto &x : stg[d][2]->v) x = inv2;
            for (auto &x : col[d][0]->v) x = inv;
            for (auto &x : col[d][1]->v) x = 0.0;
            for (auto &x : col[d][2]->v) x = inv2;
        }
        xStaggr.resize(-1, sx); yStaggr.resize(-1, sy); zStaggr.resize(-1, sz);
        xColloc.resize(-1, cx); yColloc.resize(-1, cy); zColloc.resize(-1, cz);
        for (int i = -1; i < sx + 1; i++) xStaggr(i) = xLen * xi(i);          // grid.cc:374-376
        for (int i = -1; i < cx + 1; i++) xColloc(i) = xLen * (xi(i) + xi(i + 1)) / 2.0;
        for (int i = -1; i < sy + 1; i++) yStaggr(i) = yLen * et(i);
        for (int i = -1; i < cy + 1; i++) yColloc(i) = yLen * (et(i) + et(i + 1)) / 2.0;
        for (int i = -1; i < sz + 1; i++) zStaggr(i) = zLen * zt(i);
        for (int i = -1; i < cz + 1; i++) zColloc(i) = zLen * (zt(i) + zt(i + 1)) / 2.0;
        // grid.cc:117-131 with createTanHypGrid (grid.cc:442-519): on the axes
        // whose mesh type is 'D' (xGrid = 2) the core coordinates and metrics
        // are replaced by the double-sided tangent-hyperbolic map; the ghost
        // entries keep their uniform values.
        const int gtype[3] = {p.xGrid, p.yGrid, p.zGrid};
        const double beta[3] = {p.betaX, p.betaY, p.betaZ};
        const A1 *tc[3] = {&xi, &et, &zt};
        A1 *sco[3] = {&xStaggr, &yStaggr, &zStaggr}, *cco[3] = {&xColloc, &yColloc, &zColloc};
        for (int d = 0; d < 3; ++d) {
            if (gtype[d] != 2 || (planar && d == 1)) continue;
            const double b = beta[d], Ld = L[d];
            const A1 &t = *tc[d];
            auto metrics = [&](A1 *const m[3], int i, double x) {
                (*m[0])(i) = std::tanh(b) / (b * Ld * (1.0 - std::pow((1.0 - 2.0 * x / Ld) * std::tanh(b), 2)));
                (*m[1])(i) = -4.0 * std::pow(std::tanh(b), 3) * (1.0 - 2.0 * x / Ld) /
                             (b * Ld * Ld * std::pow(1.0 - std::pow(std::tanh(b) * (1.0 - 2.0 * x / Ld), 2), 2));
                (*m[2])(i) = std::pow((*m[0])(i), 2.0);
            };
            for (int i = 0; i < sc[d]; i++) {
                (*sco[d])(i) = Ld * (1.0 - std::tanh(b * (1.0 - 2.0 * t(i))) / std::tanh(b)) / 2.0;
                metrics(stg[d], i, (*sco[d])(i));
            }
            for (int i = 0; i < cc[d]; i++) {
                (*cco[d])(i) = Ld * (1.0 - std::tanh(b * (1.0 - (t(i) + t(i + 1)))) / std::tanh(b)) / 2.0;
                metrics(col[d], i, (*cco[d])(i));
            }
        }
    }
};

// ------------------------------------------------------------------ fields
// field.cc:66-290: storage, core, bulk and wall slices of a field at np = 1.
struct Field {
    bool stag[3];
    int cnt[3];          // core count along each axis (cuBound + 1)
    int blb[3], bub[3];  // bulk bounds
    A3 F;
    void build(const Grid &g, const saras_params &p, bool xs, bool ys, bool zs) {
        stag[0] = xs; stag[1] = ys; stag[2] = zs;
        bool per[3] = {p.xPer != 0, p.yPer != 0, p.zPer != 0};
        for (int d = 0; d < 3; ++d) {
            cnt[d] = stag[d] ? g.staggrCoreSize[d] : g.collocCoreSize[d];
            blb[d] = 0; bub[d] = cnt[d] - 1;
            if (stag[d] && !per[d]) { blb[d] += 1; bub[d] -= 1; }   // field.cc:206-219
        }
        if (g.planar) { blb[1] = 0; bub[1] = 0; }   // field.cc:221-224
        F.resize(-1, -1, -1, cnt[0], cnt[1], cnt[2]);
    }
    int w0(int d) const { return blb[d] - 1; }   // field.cc:269-285
    int w1(int d) const { return bub[d] + 1; }
};

// mpidata::syncData at np = 1 (mpidata.cc:82-306): periodic face copies over
// the core range of the other two axes, then the four x-y edge copies over the
// core z range.  Edge neighbours are always periodic (parallel.cc:124-130) and
// are never reset by hydro::checkPeriodic (hydro.cc:174-212).
static void syncData(A3 &F, const Field &f, bool xPer, bool yPer, bool planar = false) {
    int cx = f.cnt[0], cy = f.cnt[1], cz = f.cnt[2];
    int lsx = f.stag[0] ? 1 : 0, hsx = cx - 1 - (f.stag[0] ? 1 : 0);
    int lsy = f.stag[1] ? 1 : 0, hsy = cy - 1 - (f.stag[1] ? 1 : 0);
    if (xPer) {
        for (int j = 0; j < cy; ++j) for (int k = 0; k < cz; ++k) {
            F(-1, j, k) = F(hsx, j, k);
            F(cx, j, k) = F(lsx, j, k);
        }
    }
    // 2D: no y neighbours and no edge neighbours (parallel.cc:118-130, hydro.cc:188-191)
    if (planar) return;
    if (yPer) {
        for (int i = 0; i < cx; ++i) for (int k = 0; k < cz; ++k) {
            F(i, -1, k) = F(i, hsy, k);
            F(i, cy, k) = F(i, lsy, k);
        }
    }
    for (int k = 0; k < cz; ++k) {
        F(-1, -1, k) = F(hsx, hsy, k);
        F(-1, cy, k) = F(hsx, lsy, k);
        F(cx, -1, k) = F(lsx, hsy, k);
        F(cx, cy, k) = F(lsx, lsy, k);
    }
}

// ------------------------------------------------------------------ boundary
// boundary.cc:57-91 and the subclasses of lib/boundary.
enum BCType { BC_NULL, BC_DIR_CC, BC_DIR_FC, BC_NEU_CC, BC_NEU_FC, BC_PER_CC, BC_PER_FC };
struct BC { BCType t = BC_NULL; int wall = 0; double v = 0.0; };

// Iterate over a wall slice (field.cc:249-290): the wall index along its axis,
// the full padded range along the other two.
template <class Fn>
static void forWall(const Field &f, int wall, int windex, Fn fn) {
    int dim = wall / 2;
    int lo[3] = {-1, -1, -1}, hi[3] = {f.cnt[0], f.cnt[1], f.cnt[2]};
    lo[dim] = hi[dim] = windex;
    for (int i = lo[0]; i <= hi[0]; ++i) for (int j = lo[1]; j <= hi[1]; ++j) for (int k = lo[2]; k <= hi[2]; ++k) fn(i, j, k);
}

static void imposeBC(Field &f, const BC &bc) {
    int dim = bc.wall / 2;
    int shiftVal = (bc.wall % 2 == 0) ? 1 : -1;   // boundary.cc:66-87
    int windex = (bc.wall % 2 == 0) ? f.w0(dim) : f.w1(dim);
    A3 &F = f.F;
    auto at = [&](int i, int j, int k, int off) -> double & {
        int ii = i, jj = j, kk = k;
        if (dim == 0) ii += off; else if (dim == 1) jj += off; else kk += off;
        return F(ii, jj, kk);
    };
    switch (bc.t) {
    case BC_NULL: break;
    case BC_DIR_CC:   // dirichletCC.cc:71-75
        forWall(f, bc.wall, windex, [&](int i, int j, int k) { F(i, j, k) = bc.v; });
        break;
    case BC_DIR_FC:   // dirichletFC.cc:71-75
        forWall(f, bc.wall, windex, [&](int i, int j, int k) { F(i, j, k) = 2.0 * bc.v - at(i, j, k, shiftVal); });
        break;
    case BC_NEU_CC:   // neumannCC.cc:71-79
    case BC_NEU_FC:   // neumannFC.cc:71-76
        forWall(f, bc.wall, windex, [&](int i, int j, int k) { F(i, j, k) = at(i, j, k, shiftVal); });
        break;
    case BC_PER_CC: { // periodicCC.cc:72-83
        int src = (shiftVal > 0) ? f.w1(dim) - 2 : f.w0(dim) + 2;
        forWall(f, bc.wall, windex, [&](int i, int j, int k) { F(i, j, k) = at(i, j, k, src - windex); });
        break;
    }
    case BC_PER_FC: { // periodicFC.cc:72-81
        int src = (shiftVal > 0) ? f.w1(dim) - 1 : f.w0(dim) + 1;
        forWall(f, bc.wall, windex, [&](int i, int j, int k) { F(i, j, k) = at(i, j, k, src - windex); });
        break;
    }
    }
}

// ------------------------------------------------------------------ multigrid
// poisson.cc / poisson_d3.cc at np = 1.
struct Multigrid {
    const Grid *g = nullptr;
    saras_params p{};
    int d = 0;
    std::vector<A3> pressureData, residualData, tmpDataArray, smoothedPres;
    std::vector<int> xEnd, yEnd, zEnd, strideValues;
    std::vector<double> hx, hy, hz, hxhy, hyhz, hzhx, hxhyhz;
    std::vector<double> hx2, hz2;   // 2D (poisson.cc:406-409, 426-428)
    bool planar = false;
    std::vector<A1> xixx, xix2, etyy, ety2, ztzz, ztz2;
    int vLevel = 0, maxCount = 0;
    bool zeroBC = false;
    A3 xWall, yWall, zWall;   // 2D walls stored with a unit third axis
    long long coarseIters = 0;

    void build(const Grid &grid, const saras_params &prm) {
        g = &grid; p = prm; d = p.vcDepth;
        strideValues.resize(d + 1);
        for (int i = 0; i <= d; i++) strideValues[i] = int(std::pow(2, i));          // poisson.cc:74-77
        xEnd.resize(d + 1); yEnd.resize(d + 1); zEnd.resize(d + 1);
        for (int i = 0; i <= d; i++) {                                               // poisson.cc:336-357
            xEnd[i] = int(std::pow(2, g->sizeIndex[0] - i));
            yEnd[i] = int(std::pow(2, g->sizeIndex[1] - i));
            zEnd[i] = int(std::pow(2, g->sizeIndex[2] - i));
            if (g->planar) yEnd[i] = 0;   // poisson.cc:339-340: one y point on every level
        }
        planar = g->planar;
        maxCount = (xEnd[d] + 2) * (yEnd[d] + 2) * (zEnd[d] + 2);                    // poisson.cc:360-361
        hx.resize(d + 1); hy.resize(d + 1); hz.resize(d + 1);
        hxhy.resize(d + 1); hyhz.resize(d + 1); hzhx.resize(d + 1); hxhyhz.resize(d + 1);
        for (int i = 0; i <= d; i++) {                                               // poisson.cc:419-438
            hx[i] = strideValues[i] * g->dXi;
            hy[i] = strideValues[i] * g->dEt;
            hz[i] = strideValues[i] * g->dZt;
            hxhy[i] = std::pow(strideValues[i], 4.0) * std::pow(g->dXi, 2.0) * std::pow(g->dEt, 2.0);
            hyhz[i] = std::pow(strideValues[i], 4.0) * std::pow(g->dEt, 2.0) * std::pow(g->dZt, 2.0);
            hzhx[i] = std::pow(strideValues[i], 4.0) * std::pow(g->dZt, 2.0) * std::pow(g->dXi, 2.0);
            hxhyhz[i] = std::pow(strideValues[i], 6.0) * std::pow(g->dXi, 2.0) * std::pow(g->dEt, 2.0) * std::pow(g->dZt, 2.0);
        }
        hx2.resize(d + 1); hz2.resize(d + 1);
        for (int i = 0; i <= d; i++) {
            hx2[i] = std::pow(strideValues[i] * g->dXi, 2.0);
            hz2[i] = std::pow(strideValues[i] * g->dZt, 2.0);
        }
        xixx.resize(d + 1); xix2.resize(d + 1); etyy.resize(d + 1); ety2.resize(d + 1); ztzz.resize(d + 1); ztz2.resize(d + 1);
        for (int n = 0; n <= d; ++n) {                                               // poisson.cc:463-495
            int s = strideValues[n];
            xixx[n].resize(-1, xEnd[n] + 1); xix2[n].resize(-1, xEnd[n] + 1);
            etyy[n].resize(-1, yEnd[n] + 1); ety2[n].resize(-1, yEnd[n] + 1);
            ztzz[n].resize(-1, zEnd[n] + 1); ztz2[n].resize(-1, zEnd[n] + 1);
            for (int i = 0; i <= xEnd[n]; ++i) { xixx[n](i) = g->xixxStaggr(i * s); xix2[n](i) = g->xix2Staggr(i * s); }
            for (int i = 0; i <= yEnd[n]; ++i) { etyy[n](i) = g->etyyStaggr(i * s); ety2[n](i) = g->ety2Staggr(i * s); }
            for (int i = 0; i <= zEnd[n]; ++i) { ztzz[n](i) = g->ztzzStaggr(i * s); ztz2[n](i) = g->ztz2Staggr(i * s); }
        }
        pressureData.resize(d + 1); residualData.resize(d + 1); tmpDataArray.resize(d + 1); smoothedPres.resize(d + 1);
        for (int i = 0; i <= d; i++) {                                               // poisson.cc:293-316
            pressureData[i].resize(-1, -1, -1, xEnd[i] + 1, yEnd[i] + 1, zEnd[i] + 1);
            residualData[i].resize(-1, -1, -1, xEnd[i] + 1, yEnd[i] + 1, zEnd[i] + 1);
            tmpDataArray[i].resize(-1, -1, -1, xEnd[i] + 1, yEnd[i] + 1, zEnd[i] + 1);
            smoothedPres[i].resize(-1, -1, -1, xEnd[i] + 1, yEnd[i] + 1, zEnd[i] + 1);
        }
        if (p.testPoisson) initDirichlet();
    }

    // poisson_d3.cc:513-572 (np = 1: halfInd = xEnd(0)/2)
    void initDirichlet() {
        int X = xEnd[0], Y = yEnd[0], Z = zEnd[0];
        xWall.resize(-1, -1, 0, Y + 1, Z + 1, 0);
        yWall.resize(-1, -1, 0, X + 1, Z + 1, 0);
        zWall.resize(-1, -1, 0, X + 1, Y + 1, 0);
        int halfIndX = X / 2, halfIndY = Y / 2;
        double xDist, yDist, zDist;
        xDist = hx[0] + p.Lx / 2.0;
        for (int j = 0; j <= Y; ++j) {
            yDist = hy[0] * (j - halfIndY);
            for (int k = 0; k <= Z; ++k) {
                zDist = hz[0] * (k - Z / 2);
                xWall(j, k, 0) = (xDist * xDist + yDist * yDist + zDist * zDist) / 6.0;
            }
        }
        yDist = hy[0] + p.Ly / 2.0;
        for (int i = 0; i <= X; ++i) {
            xDist = hx[0] * (i - halfIndX);
            for (int k = 0; k <= Z; ++k) {
                zDist = hz[0] * (k - Z / 2);
                yWall(i, k, 0) = (xDist * xDist + yDist * yDist + zDist * zDist) / 6.0;
            }
        }
        zDist = hz[0] + p.Lz / 2.0;
        for (int i = 0; i <= X; ++i) {
            xDist = hx[0] * (i - halfIndX);
            for (int j = 0; j <= Y; ++j) {
                yDist = hy[0] * (j - halfIndY);
                zWall(i, j, 0) = (xDist * xDist + yDist * yDist + zDist * zDist) / 6.0;
            }
        }
    }

    // poisson_d3.cc:671-686 at np = 1: periodic self-exchange of whole x planes,
    // then whole y planes (which include the freshly written x ghosts).
    void updatePads(std::vector<A3> &data) {
        A3 &a = data[vLevel];
        int X = xEnd[vLevel], Y = yEnd[vLevel], Z = zEnd[vLevel];
        if (p.xPer) {
            for (int j = -1; j <= Y + 1; ++j) for (int k = -1; k <= Z + 1; ++k) a(X + 1, j, k) = a(1, j, k);
            for (int j = -1; j <= Y + 1; ++j) for (int k = -1; k <= Z + 1; ++k) a(-1, j, k) = a(X - 1, j, k);
        }
        if (p.yPer && !planar) {   // 2D: no y neighbours (poisson_d2.cc updatePads exchanges x only)
            for (int i = -1; i <= X + 1; ++i) for (int k = -1; k <= Z + 1; ++k) a(i, Y + 1, k) = a(i, 1, k);
            for (int i = -1; i <= X + 1; ++i) for (int k = -1; k <= Z + 1; ++k) a(i, -1, k) = a(i, Y - 1, k);
        }
    }

    // poisson_d3.cc:575-668
    void imposeBC() {
        updatePads(pressureData);
        A3 &a = pressureData[vLevel];
        int X = xEnd[vLevel], Y = yEnd[vLevel], Z = zEnd[vLevel];
        if (!p.xPer) {
            for (int j = -1; j <= Y + 1; ++j) for (int k = -1; k <= Z + 1; ++k) {
                if (p.testPoisson) {
                    if (zeroBC) { a(-1, j, k) = -a(1, j, k); a(X + 1, j, k) = -a(X - 1, j, k); }
                    else { a(-1, j, k) = xWall(j, k, 0); a(X + 1, j, k) = xWall(j, k, 0); }
                } else {
                    a(-1, j, k) = a(1, j, k);
                    a(X + 1, j, k) = a(X - 1, j, k);
                }
            }
        }
        if (!p.yPer && !planar) {   // 2D: no y walls (poisson_d2.cc:300-361)
            for (int i = -1; i <= X + 1; ++i) for (int k = -1; k <= Z + 1; ++k) {
                if (p.testPoisson) {
                    if (zeroBC) { a(i, -1, k) = -a(i, 1, k); a(i, Y + 1, k) = -a(i, Y - 1, k); }
                    else { a(i, -1, k) = yWall(i, k, 0); a(i, Y + 1, k) = yWall(i, k, 0); }
                } else {
                    a(i, -1, k) = a(i, 1, k);
                    a(i, Y + 1, k) = a(i, Y - 1, k);
                }
            }
        }
        for (int i = -1; i <= X + 1; ++i) for (int j = -1; j <= Y + 1; ++j) {
            if (p.zPer) {
                a(i, j, -1) = a(i, j, Z - 1);
                a(i, j, Z + 1) = a(i, j, 1);
            } else if (p.testPoisson) {
                if (zeroBC) { a(i, j, -1) = -a(i, j, 1); a(i, j, Z + 1) = -a(i, j, Z - 1); }
                else { a(i, j, -1) = zWall(i, j, 0); a(i, j, Z + 1) = zWall(i, j, 0); }
            } else {
                a(i, j, -1) = a(i, j, 1);
                a(i, j, Z + 1) = a(i, j, Z - 1);
            }
        }
    }

    // Laplacian at level l, the expression of poisson_d3.cc:99-105
    // (poisson_d2.cc:97-100 in 2D).
    inline double lap(const A3 &P, int l, int i, int j, int k) const {
        if (planar)
            return xix2[l](i) * (P(i + 1, j, k) - 2.0 * P(i, j, k) + P(i - 1, j, k)) / (hx[l] * hx[l]) +
                   xixx[l](i) * (P(i + 1, j, k) - P(i - 1, j, k)) / (2.0 * hx[l]) +
                   ztz2[l](k) * (P(i, j, k + 1) - 2.0 * P(i, j, k) + P(i, j, k - 1)) / (hz[l] * hz[l]) +
                   ztzz[l](k) * (P(i, j, k + 1) - P(i, j, k - 1)) / (2.0 * hz[l]);
        return xix2[l](i) * (P(i + 1, j, k) - 2.0 * P(i, j, k) + P(i - 1, j, k)) / (hx[l] * hx[l]) +
               xixx[l](i) * (P(i + 1, j, k) - P(i - 1, j, k)) / (2.0 * hx[l]) +
               ety2[l](j) * (P(i, j + 1, k) - 2.0 * P(i, j, k) + P(i, j - 1, k)) / (hy[l] * hy[l]) +
               etyy[l](j) * (P(i, j + 1, k) - P(i, j - 1, k)) / (2.0 * hy[l]) +
               ztz2[l](k) * (P(i, j, k + 1) - 2.0 * P(i, j, k) + P(i, j, k - 1)) / (hz[l] * hz[l]) +
               ztzz[l](k) * (P(i, j, k + 1) - P(i, j, k - 1)) / (2.0 * hz[l]);
    }

    // Gauss-Seidel / Jacobi update, the expression of poisson_d3.cc:140-147
    // (poisson_d2.cc:126-131 in 2D).
    inline double update(const A3 &P, const A3 &R, int l, int i, int j, int k) const {
        if (planar)
            return (hz2[l] * xix2[l](i) * (P(i + 1, j, k) + P(i - 1, j, k)) * 2.0 +
                    hz2[l] * xixx[l](i) * (P(i + 1, j, k) - P(i - 1, j, k)) * hx[l] +
                    hx2[l] * ztz2[l](k) * (P(i, j, k + 1) + P(i, j, k - 1)) * 2.0 +
                    hx2[l] * ztzz[l](k) * (P(i, j, k + 1) - P(i, j, k - 1)) * hz[l] -
                    2.0 * hzhx[l] * R(i, j, k)) /
                   (4.0 * (hz2[l] * xix2[l](i) + hx2[l] * ztz2[l](k)));
        return (hyhz[l] * xix2[l](i) * (P(i + 1, j, k) + P(i - 1, j, k)) * 2.0 +
                hyhz[l] * xixx[l](i) * (P(i + 1, j, k) - P(i - 1, j, k)) * hx[l] +
                hzhx[l] * ety2[l](j) * (P(i, j + 1, k) + P(i, j - 1, k)) * 2.0 +
                hzhx[l] * etyy[l](j) * (P(i, j + 1, k) - P(i, j - 1, k)) * hy[l] +
                hxhy[l] * ztz2[l](k) * (P(i, j, k + 1) + P(i, j, k - 1)) * 2.0 +
                hxhy[l] * ztzz[l](k) * (P(i, j, k + 1) - P(i, j, k - 1)) * hz[l] -
                2.0 * hxhyhz[l] * R(i, j, k)) /
               (4.0 * (hyhz[l] * xix2[l](i) + hzhx[l] * ety2[l](j) + hxhy[l] * ztz2[l](k)));
    }

    // poisson_d3.cc:90-111
    void computeResidual() {
        int l = vLevel;
        tmpDataArray[l].fill(0.0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i <= xEnd[l]; ++i) for (int j = 0; j <= yEnd[l]; ++j) for (int k = 0; k <= zEnd[l]; ++k)
            tmpDataArray[l](i, j, k) = residualData[l](i, j, k) - lap(pressureData[l], l, i, j, k);
        updatePads(tmpDataArray);
    }

    // poisson_d3.cc:114-187.  Blitz's swap(Array&, Array&) exchanges the two
    // level vectors by reference, so std::swap of the vectors is exact.
    void smooth(int smoothCount) {
        int l = vLevel;
        tmpDataArray[l].fill(0.0);
        for (int n = 0; n < smoothCount; ++n) {
            imposeBC();
            if (p.gsSmooth) {
                A3 &P = pressureData[l];
                for (int i = 0; i <= xEnd[l]; ++i) for (int j = 0; j <= yEnd[l]; ++j) for (int k = 0; k <= zEnd[l]; ++k)
                    P(i, j, k) = update(P, residualData[l], l, i, j, k);
            } else {
#pragma omp parallel for schedule(static)
                for (int i = 0; i <= xEnd[l]; ++i) for (int j = 0; j <= yEnd[l]; ++j) for (int k = 0; k <= zEnd[l]; ++k)
                    tmpDataArray[l](i, j, k) = update(pressureData[l], residualData[l], l, i, j, k);
                std::swap(tmpDataArray, pressureData);
            }
        }
        imposeBC();
    }

    // poisson_d3.cc:190-247
    void solve() {
        int l = vLevel;
        int iterCount = 0;
        double tempValue, localMax, globalMax;
        while (true) {
            imposeBC();
            A3 &P = pressureData[l];
            for (int i = 0; i <= xEnd[l]; ++i) for (int j = 0; j <= yEnd[l]; ++j) for (int k = 0; k <= zEnd[l]; ++k)
                P(i, j, k) = update(P, residualData[l], l, i, j, k);
            coarseIters += 1;
            tempValue = 0.0;
            localMax = -1.0e-10;
            for (int i = 0; i <= xEnd[l]; ++i) for (int j = 0; j <= yEnd[l]; ++j) for (int k = 0; k <= zEnd[l]; ++k) {
                tempValue = std::fabs(residualData[l](i, j, k) - lap(P, l, i, j, k));
                if (tempValue > localMax) localMax = tempValue;
            }
            globalMax = localMax;
            if (globalMax < p.mgTolerance) break;
            iterCount += 1;
            if (iterCount > maxCount) break;
        }
        imposeBC();
    }

    // poisson_d3.cc:250-298
    void coarsen() {
        int pLevel = vLevel;
        vLevel += 1;
        const A3 &T = tmpDataArray[pLevel];
        A3 &R = residualData[vLevel];
        if (planar) {   // poisson_d2.cc:207-225: 9-point full weighting in the y = 0 plane
            for (int i = 0; i <= xEnd[vLevel]; ++i) {
                int i2 = i * 2;
                for (int k = 0; k <= zEnd[vLevel]; ++k) {
                    int k2 = k * 2;
                    double facePoints = (T(i2 + 1, 0, k2) + T(i2 - 1, 0, k2) + T(i2, 0, k2 + 1) + T(i2, 0, k2 - 1)) * 0.125;
                    double vertPoints = (T(i2 + 1, 0, k2 + 1) + T(i2 + 1, 0, k2 - 1) + T(i2 - 1, 0, k2 + 1) + T(i2 - 1, 0, k2 - 1)) * 0.0625;
                    R(i, 0, k) = facePoints + vertPoints + T(i2, 0, k2) * 0.25;
                }
            }
            return;
        }
#pragma omp parallel for schedule(static)
        for (int i = 0; i <= xEnd[vLevel]; ++i) {
            int i2 = i * 2;
            for (int j = 0; j <= yEnd[vLevel]; ++j) {
                int j2 = j * 2;
                for (int k = 0; k <= zEnd[vLevel]; ++k) {
                    int k2 = k * 2;
                    double facePoints = (T(i2 + 1, j2, k2) + T(i2 - 1, j2, k2) +
                                         T(i2, j2 + 1, k2) + T(i2, j2 - 1, k2) +
                                         T(i2, j2, k2 + 1) + T(i2, j2, k2 - 1)) * 0.0625;
                    double edgePoints = (T(i2 + 1, j2 + 1, k2) + T(i2 + 1, j2 - 1, k2) +
                                         T(i2 - 1, j2 - 1, k2) + T(i2 - 1, j2 + 1, k2) +
                                         T(i2, j2 + 1, k2 + 1) + T(i2, j2 - 1, k2 + 1) +
                                         T(i2, j2 - 1, k2 - 1) + T(i2, j2 + 1, k2 - 1) +
                                         T(i2 + 1, j2, k2 + 1) + T(i2 + 1, j2, k2 - 1) +
                                         T(i2 - 1, j2, k2 - 1) + T(i2 - 1, j2, k2 + 1)) * 0.03125;
                    double vertPoints = (T(i2 + 1, j2 + 1, k2 + 1) +
                                         T(i2 + 1, j2 + 1, k2 - 1) +
                                         T(i2 + 1, j2 - 1, k2 + 1) +
                                         T(i2 - 1, j2 + 1, k2 + 1) +
                                         T(i2 + 1, j2 - 1, k2 - 1) +
                                         T(i2 - 1, j2 + 1, k2 - 1) +
                                         T(i2 - 1, j2 - 1, k2 + 1) +
                                         T(i2 - 1, j2 - 1, k2 - 1)) * 0.015625;
                    R(i, j, k) = facePoints + edgePoints + vertPoints + T(i2, j2, k2) * 0.125;
                }
            }
        }
    }

    // poisson_d3.cc:301-388
    void prolong() {
        int pLevel = vLevel;
        vLevel -= 1;
        A3 &F = pressureData[vLevel];
        const A3 &C = pressureData[pLevel];
        F.fill(0.0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i <= xEnd[vLevel]; ++i) {
            int i2 = i / 2;
            for (int j = 0; j <= yEnd[vLevel]; ++j) {
                int j2 = j / 2;
                for (int k = 0; k <= zEnd[vLevel]; ++k) {
                    int k2 = k / 2;
                    bool io = i % 2, jo = j % 2, ko = k % 2;
                    double v;
                    if (io) {
                        if (jo) {
                            if (ko) v = (C(i2, j2, k2) + C(i2 + 1, j2, k2) + C(i2, j2 + 1, k2) + C(i2, j2, k2 + 1) +
                                         C(i2 + 1, j2 + 1, k2) + C(i2 + 1, j2, k2 + 1) + C(i2, j2 + 1, k2 + 1) +
                                         C(i2 + 1, j2 + 1, k2 + 1)) / 8.0;
                            else v = (C(i2, j2, k2) + C(i2, j2 + 1, k2) + C(i2 + 1, j2, k2) + C(i2 + 1, j2 + 1, k2)) / 4.0;
                        } else {
                            if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1) + C(i2 + 1, j2, k2) + C(i2 + 1, j2, k2 + 1)) / 4.0;
                            else v = (C(i2, j2, k2) + C(i2 + 1, j2, k2)) / 2.0;
                        }
                    } else {
                        if (jo) {
                            if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1) + C(i2, j2 + 1, k2) + C(i2, j2 + 1, k2 + 1)) / 4.0;
                            else v = (C(i2, j2, k2) + C(i2, j2 + 1, k2)) / 2.0;
                        } else {
                            if (ko) v = (C(i2, j2, k2) + C(i2, j2, k2 + 1)) / 2.0;
                            else v = C(i2, j2, k2);
                        }
                    }
                    F(i, j, k) = v;
                }
            }
        }
    }

    // poisson_d3.cc:391-459
    double computeError(int normOrder) {
        double residualVal = 0.0, tempValue = 0.0, numValLoc = 0.0, denValLoc = 0.0;
        int valCountLoc = 0;
        const A3 &P = pressureData[0];
        const A3 &R = residualData[0];
        int X = xEnd[0], Y = yEnd[0], Z = zEnd[0];
        long ncore = (long)(X + 1) * (Y + 1) * (Z + 1);
        auto pt = [&](long t, int &i, int &j, int &k) { k = (int)(t % (Z + 1)); j = (int)((t / (Z + 1)) % (Y + 1)); i = (int)(t / ((long)(Z + 1) * (Y + 1))); };
        if (normOrder == 1) {
#pragma omp parallel for schedule(static) reduction(max : numValLoc) private(tempValue)
            for (int i = 0; i <= X; ++i) for (int j = 0; j <= Y; ++j) for (int k = 0; k <= Z; ++k) {
                // hx(vLevel) with vLevel = 0 at this point
                tempValue = std::fabs(lap(P, 0, i, j, k) - R(i, j, k));
                if (tempValue > numValLoc) numValLoc = tempValue;
            }
        } else if (normOrder == 2) {
            // sums in the chunked order shared with the GPU (see chunked_sum)
            numValLoc = chunked_sum(ncore, [&](long t) { int i, j, k; pt(t, i, j, k); double v = std::fabs(lap(P, 0, i, j, k) - R(i, j, k)); return v * v; });
            denValLoc = chunked_sum(ncore, [&](long t) { int i, j, k; pt(t, i, j, k); return R(i, j, k) * R(i, j, k); });
            valCountLoc = (int)ncore;
        }
        switch (normOrder) {
        case 1: {
            denValLoc = 0.0;  // blitz::max(fabs(residualData(0))) over the padded array
            for (double x : R.v) { double a = std::fabs(x); if (a > denValLoc) denValLoc = a; }
            residualVal = denValLoc ? numValLoc / denValLoc : numValLoc;
            break;
        }
        case 2:
            residualVal = denValLoc ? std::sqrt(numValLoc / valCountLoc) / std::sqrt(denValLoc / valCountLoc)
                                    : std::sqrt(numValLoc / valCountLoc);
            break;
        }
        return residualVal;
    }

    // poisson.cc:219-280
    void vCycle() {
        vLevel = 0;
        zeroBC = false;
        smooth(p.preSmooth);
        zeroBC = true;
        for (int i = 0; i < d; i++) {
            computeResidual();
            smoothedPres[vLevel] = pressureData[vLevel];
            coarsen();
            pressureData[vLevel].fill(0.0);
            if (vLevel == d) solve(); else smooth(p.preSmooth);
        }
        for (int i = 0; i < d; i++) {
            prolong();
            A3 &P = pressureData[vLevel];
            const A3 &S = smoothedPres[vLevel];
            for (size_t n = 0; n < P.v.size(); ++n) P.v[n] += S.v[n];
            zeroBC = (vLevel != 0);
            smooth(p.postSmooth);
        }
    }

    // poisson.cc:100-205.  Returns the number of V-cycles performed.
    int mgSolve(A3 &inFn, const A3 &rhs, double *lastResidual) {
        double prevResidual = 0.0;
        vLevel = 0;
        for (int i = 0; i <= d; i++) {
            pressureData[i].fill(0.0); residualData[i].fill(0.0); smoothedPres[i].fill(0.0);
        }
        for (int i = 0; i <= xEnd[0]; ++i) for (int j = 0; j <= yEnd[0]; ++j) for (int k = 0; k <= zEnd[0]; ++k) {
            residualData[0](i, j, k) = rhs(i, j, k);
            pressureData[0](i, j, k) = inFn(i, j, k);
        }
        updatePads(residualData);
        updatePads(pressureData);
        if (!p.testPoisson) {
            // blitz::mean over the padded array: sum / count (chunked order)
            const std::vector<double> &rv = residualData[0].v;
            double s = chunked_sum((long)rv.size(), [&](long t) { return rv[(size_t)t]; });
            double localMean = s / double(residualData[0].v.size());
            double globalAvg = localMean / 1.0;   // MPI_Allreduce / nProc at np = 1
            for (double &x : residualData[0].v) x -= globalAvg;
        }
        int cycles = 0;
        double mgResidual = 0.0;
        for (int i = 0; i < p.vcCount; i++) {
            vCycle();
            cycles += 1;
            mgResidual = computeError(p.resType);
            if (!p.testPoisson) {
                if (std::fabs(prevResidual - mgResidual) < p.mgTolerance) break;
                prevResidual = mgResidual;
            }
        }
        if (lastResidual) *lastResidual = mgResidual;
        inFn.v = pressureData[0].v;   // poisson.cc:151: whole padded array
        return cycles;
    }

    // poisson_d3.cc:689-719
    double testProlong() {
        vLevel = 0;
        residualData[vLevel].fill(0.0);
        for (int i = 0; i <= xEnd[vLevel]; ++i) for (int j = 0; j <= yEnd[vLevel]; ++j) for (int k = 0; k <= zEnd[vLevel]; ++k)
            residualData[vLevel](i, j, k) = (0 + 1) * 1000 + i * 100 + j * 10 + k;
        vLevel += 1;
        pressureData[vLevel].fill(0.0);
        // The reference fills the coarse level with coarse indices, a field
        // that prolongation cannot reproduce; the restatement samples the same
        // linear function at the coincident fine indices (2i, 2j, 2k), which
        // trilinear prolongation must reproduce exactly.
        for (int i = 0; i <= xEnd[vLevel]; ++i) for (int j = 0; j <= yEnd[vLevel]; ++j) for (int k = 0; k <= zEnd[vLevel]; ++k)
            pressureData[vLevel](i, j, k) = (0 + 1) * 1000 + (2 * i) * 100 + (2 * j) * 10 + (2 * k);
        prolong();
        double m = 0.0;
        A3 &P = pressureData[vLevel];
        const A3 &R = residualData[vLevel];
        for (size_t n = 0; n < P.v.size(); ++n) { P.v[n] -= R.v[n]; m = std::max(m, std::fabs(P.v[n])); }
        return m;
    }

    // poisson_d3.cc:722-777 at np = 1 (faceRanks = 0 when periodic, PROC_NULL otherwise).
    // With non-periodic x/y the pads are not exchanged, so the expected values
    // (built from faceRanks = MPI_PROC_NULL) do not apply; the reference test
    // is only meaningful for periodic x and y, which is what it is called with.
    double testTransfer() {
        double maxVal = 0.0;
        vLevel = 0;
        pressureData[vLevel].fill(0.0);
        residualData[vLevel].fill(0.0);
        for (int i = 0; i <= xEnd[vLevel]; ++i) for (int j = 0; j <= yEnd[vLevel]; ++j) for (int k = 0; k <= zEnd[vLevel]; ++k) {
            pressureData[vLevel](i, j, k) = (0 + 1) * 1000 + i * 100 + j * 10 + k;
            residualData[vLevel](i, j, k) = pressureData[vLevel](i, j, k);
        }
        const int fr = 0;  // self
        for (int n = 0; n <= d; n++) for (int j = 0; j <= yEnd[n]; ++j) for (int k = 0; k <= zEnd[n]; ++k) {
            residualData[n](-1, j, k) = (fr + 1) * 1000 + (xEnd[n] - 1) * 100 + j * 10 + k;
            residualData[n](xEnd[n] + 1, j, k) = (fr + 1) * 1000 + 100 + j * 10 + k;
        }
        for (int n = 0; n <= d; n++) for (int i = 0; i <= xEnd[n]; ++i) for (int k = 0; k <= zEnd[n]; ++k) {
            residualData[n](i, -1, k) = (fr + 1) * 1000 + i * 100 + (yEnd[n] - 1) * 10 + k;
            residualData[n](i, yEnd[n] + 1, k) = (fr + 1) * 1000 + i * 100 + 10 + k;
        }
        for (int n = 0; n <= d; n++) { updatePads(pressureData); vLevel += 1; }
        // vLevel == d + 1 here in the reference (poisson_d3.cc:764) -- an index
        // one past the hierarchy; the comparison is done at level 0, the only
        // level whose pressure data was filled, over the core and the face
        // pads (the x-y corner pads of the expected array are never set by
        // the reference, poisson_d3.cc:741-757).
        int l = 0;
        A3 &P = pressureData[l];
        const A3 &R = residualData[l];
        for (int i = P.lb[0]; i <= P.ub[0]; i++) for (int j = P.lb[1]; j <= P.ub[1]; j++) for (int k = 0; k <= zEnd[l]; k++) {
            if ((i < 0 || i > xEnd[l]) && (j < 0 || j > yEnd[l])) continue;
            double v = P(i, j, k) - R(i, j, k);
            if (std::fabs(v) > maxVal) maxVal = std::fabs(v);
        }
        vLevel = 0;
        return maxVal;
    }

    // poisson_d3.cc:780-857 (same level-index remark as testTransfer).
    double testPeriodic() {
        double xCoord, yCoord, zCoord;
        pressureData[0].fill(0.0);
        residualData[0].fill(0.0);
        const double PI = M_PI;
        for (int i = 0; i <= xEnd[0]; ++i) for (int j = 0; j <= yEnd[0]; ++j) for (int k = 0; k <= zEnd[0]; ++k) {
            pressureData[0](i, j, k) = std::sin(2.0 * PI * g->xStaggr(i) / g->xLen) *
                                       std::cos(2.0 * PI * g->yStaggr(j) / g->yLen) *
                                       std::cos(2.0 * PI * g->zStaggr(k) / g->zLen);
            residualData[0](i, j, k) = pressureData[0](i, j, k);
        }
        for (int n = 0; n <= 0; n++) for (int j = 0; j <= yEnd[n]; ++j) for (int k = 0; k <= zEnd[n]; ++k) {
            xCoord = g->xStaggr(0) - (g->xStaggr(strideValues[n]) - g->xStaggr(0));
            residualData[n](-1, j, k) = std::sin(2.0 * PI * xCoord / g->xLen) * std::cos(2.0 * PI * g->yStaggr(j) / g->yLen) *
                                        std::cos(2.0 * PI * g->zStaggr(k) / g->zLen);
            xCoord = g->xStaggr(xEnd[0]) + (g->xStaggr(xEnd[0]) - g->xStaggr(xEnd[0] - strideValues[n]));
            residualData[n](xEnd[n] + 1, j, k) = std::sin(2.0 * PI * xCoord / g->xLen) * std::cos(2.0 * PI * g->yStaggr(j) / g->yLen) *
                                                 std::cos(2.0 * PI * g->zStaggr(k) / g->zLen);
        }
        for (int n = 0; n <= 0; n++) for (int i = 0; i <= xEnd[n]; ++i) for (int k = 0; k <= zEnd[n]; ++k) {
            yCoord = g->yStaggr(0) - (g->yStaggr(strideValues[n]) - g->yStaggr(0));
            residualData[n](i, -1, k) = std::sin(2.0 * PI * g->xStaggr(i) / g->xLen) * std::cos(2.0 * PI * yCoord / g->yLen) *
                                        std::cos(2.0 * PI * g->zStaggr(k) / g->zLen);
            yCoord = g->yStaggr(yEnd[0]) + (g->yStaggr(yEnd[0]) - g->yStaggr(yEnd[0] - strideValues[n]));
            residualData[n](i, yEnd[n] + 1, k) = std::sin(2.0 * PI * g->xStaggr(i) / g->xLen) * std::cos(2.0 * PI * yCoord / g->yLen) *
                                                 std::cos(2.0 * PI * g->zStaggr(k) / g->zLen);
        }
        for (int n = 0; n <= 0; n++) for (int i = 0; i <= xEnd[n]; ++i) for (int j = 0; j <= yEnd[n]; ++j) {
            zCoord = g->zStaggr(0) - (g->zStaggr(strideValues[n]) - g->zStaggr(0));
            residualData[n](i, j, -1) = std::sin(2.0 * PI * g->xStaggr(i) / g->xLen) * std::cos(2.0 * PI * g->yStaggr(j) / g->yLen) *
                                        std::cos(2.0 * PI * zCoord / g->zLen);
            zCoord = g->zStaggr(zEnd[0]) + (g->zStaggr(zEnd[0]) - g->zStaggr(zEnd[0] - strideValues[n]));
            residualData[n](i, j, zEnd[n] + 1) = std::sin(2.0 * PI * g->xStaggr(i) / g->xLen) * std::cos(2.0 * PI * g->yStaggr(j) / g->yLen) *
                                                 std::cos(2.0 * PI * zCoord / g->zLen);
        }
        vLevel = 0;
        imposeBC();
        // Compare the level-0 core and face ghosts (edges/corners of the
        // expected array were left at 0 by the reference and are skipped).
        double m = 0.0;
        const A3 &P = pressureData[0];
        const A3 &R = residualData[0];
        for (int i = -1; i <= xEnd[0] + 1; ++i) for (int j = -1; j <= yEnd[0] + 1; ++j) for (int k = -1; k <= zEnd[0] + 1; ++k) {
            int ng = (i < 0 || i > xEnd[0]) + (j < 0 || j > yEnd[0]) + (k < 0 || k > zEnd[0]);
            if (ng > 1) continue;
            m = std::max(m, std::fabs(P(i, j, k) - R(i, j, k)));
        }
        return m;
    }
};

// ------------------------------------------------------------------ solver
enum { VX = 0, VY = 1, VZ = 2, PF = 3, TF = 4 };

struct Solver {
    saras_params p{};
    Grid g;
    Field fx, fy, fz, fp, ft;       // V.Vx, V.Vy, V.Vz, P.F, T.F
    A3 Pp, mgRHS, nseX, nseY, nseZ, tmpRHS, gradX, gradY, gradZ;
    A3 lapX, lapY, lapZ, guessX, guessY, guessZ, guessT, lapT;
    std::vector<BC> bcs[5];         // wall objects of fx, fy, fz, -, ft (imposition order)
    Multigrid mg;
    bool isScalar = false;
    double inverseRe = 0, nu = 0, kappa = 0, Fb = 0;
    double hx, hy, hz, hz2hx2, hx2hy2, hy2hz2, hx2hy2hz2;
    double hx2 = 0, hz2 = 0;   // 2D (hydro.cc:229-232)
    int maxIterations = 0;
    double dt = 0;
    double totalVol = 0;

    Field &fieldOf(int c) { return c == VX ? fx : c == VY ? fy : c == VZ ? fz : c == PF ? fp : ft; }

    void build(const saras_params &prm) {
        p = prm;
        g.build(p);
        fx.build(g, p, false, true, true);   // vfield.cc:64-66
        fy.build(g, p, true, false, true);
        fz.build(g, p, true, true, false);
        fp.build(g, p, true, true, true);    // sfield.cc:64
        ft.build(g, p, true, true, true);
        auto like = [](A3 &a, const Field &f) { a.resize(-1, -1, -1, f.cnt[0], f.cnt[1], f.cnt[2]); };
        like(Pp, fp); like(mgRHS, fp); like(tmpRHS, fp); like(guessT, fp); like(lapT, fp);
        like(nseX, fx); like(nseY, fy); like(nseZ, fz);
        like(gradX, fx); like(gradY, fy); like(gradZ, fz);
        like(lapX, fx); like(lapY, fy); like(lapZ, fz);
        like(guessX, fx); like(guessY, fy); like(guessZ, fz);
        isScalar = (p.probType >= 5);
        inverseRe = 1.0 / p.Re;                                  // hydro.cc:65
        if (isScalar) {                                          // scalar.cc:72-89
            if (p.rbcType == 1) { nu = p.Pr; kappa = 1.0; }
            else if (p.rbcType == 2) { nu = std::sqrt(p.Pr / p.Ra); kappa = 1.0 / std::sqrt(p.Pr * p.Ra); }
            else if (p.rbcType == 3) { nu = 1.0; kappa = 1.0 / p.Pr; }
            else { nu = std::sqrt(p.Pr / p.Ra); kappa = 1.0 / std::sqrt(p.Pr * p.Ra); }
            switch (p.rbcType) {                                 // buoyantForce.cc:46-55
            case 1: Fb = p.Ra * p.Pr; break;
            case 2: Fb = 1.0; break;
            case 3: Fb = p.Ra; break;
            case 4: Fb = p.Pr; break;
            }
        }
        maxIterations = g.collocCoreSize[0] * g.collocCoreSize[1] * g.collocCoreSize[2];   // hydro.cc:74
        // hydro::setCoefficients (hydro.cc:223-241)
        hx = g.dXi; hz = g.dZt; hy = g.dEt;
        hz2hx2 = std::pow(g.dZt, 2.0) * std::pow(g.dXi, 2.0);
        hx2hy2 = std::pow(g.dXi, 2.0) * std::pow(g.dEt, 2.0);
        hy2hz2 = std::pow(g.dEt, 2.0) * std::pow(g.dZt, 2.0);
        hx2hy2hz2 = std::pow(g.dXi, 2.0) * std::pow(g.dEt, 2.0) * std::pow(g.dZt, 2.0);
        hx2 = std::pow(g.dXi, 2.0);
        hz2 = std::pow(g.dZt, 2.0);
        dt = p.tStp;
        initVBC();
        if (isScalar) initTBC();
        mg.build(g, p);
        // tseries.cc:72-108 (np = 1)
        totalVol = 0.0;
        for (int iX = 0; iX <= fp.cnt[0] - 1; iX++) for (int iY = 0; iY <= fp.cnt[1] - 1; iY++) for (int iZ = 0; iZ <= fp.cnt[2] - 1; iZ++)
            totalVol += g.planar ? (g.dXi / g.xi_xColloc(iX)) * (g.dZt / g.zt_zColloc(iZ))   // tseries.cc:93-99
                                 : (g.dXi / g.xi_xColloc(iX)) * (g.dEt / g.et_yColloc(iY)) * (g.dZt / g.zt_zColloc(iZ));
    }

    // hydro.cc:287-371 (wall order as used by imposeU/V/WBCs: Lft, Rgt, Frn, Bak, Top, Bot)
    void initVBC() {
        for (int c = 0; c < 3; ++c) bcs[c].clear();
        auto mk = [](BCType t, int w, double v) { BC b; b.t = t; b.wall = w; b.v = v; return b; };
        std::vector<BC> &u = bcs[VX], &v = bcs[VY], &w = bcs[VZ];
        if (!p.xPer) {
            if (p.probType == 3) { u.push_back(mk(BC_DIR_FC, 0, 1.0)); u.push_back(mk(BC_NEU_FC, 1, 0.0)); }
            else { u.push_back(mk(BC_DIR_FC, 0, 0.0)); u.push_back(mk(BC_DIR_FC, 1, 0.0)); }
        }
        // 2D: no front and back walls, no Vy boundary objects (hydro.cc:298-301, 320-353)
        if (!p.yPer && !g.planar) { u.push_back(mk(BC_DIR_CC, 2, 0.0)); u.push_back(mk(BC_DIR_CC, 3, 0.0)); }
        if (p.zPer) { u.push_back(mk(BC_PER_CC, 5, 0)); u.push_back(mk(BC_PER_CC, 4, 0)); }
        else if (p.probType == 1) { u.push_back(mk(BC_DIR_CC, 5, 1.0)); u.push_back(mk(BC_DIR_CC, 4, 0.0)); }
        else { u.push_back(mk(BC_DIR_CC, 5, 0.0)); u.push_back(mk(BC_DIR_CC, 4, 0.0)); }

        if (!p.xPer && !g.planar) {
            if (p.probType == 3) { v.push_back(mk(BC_DIR_CC, 0, 0.0)); v.push_back(mk(BC_NEU_CC, 1, 0.0)); }
            else { v.push_back(mk(BC_DIR_CC, 0, 0.0)); v.push_back(mk(BC_DIR_CC, 1, 0.0)); }
        }
        if (!g.planar) {
            if (!p.yPer) { v.push_back(mk(BC_DIR_FC, 2, 0.0)); v.push_back(mk(BC_DIR_FC, 3, 0.0)); }
            if (p.zPer) { v.push_back(mk(BC_PER_CC, 5, 0)); v.push_back(mk(BC_PER_CC, 4, 0)); }
            else { v.push_back(mk(BC_DIR_CC, 5, 0.0)); v.push_back(mk(BC_DIR_CC, 4, 0.0)); }
        }

        if (!p.xPer) {
            if (p.probType == 3) { w.push_back(mk(BC_DIR_CC, 0, 0.0)); w.push_back(mk(BC_NEU_CC, 1, 0.0)); }
            else { w.push_back(mk(BC_DIR_CC, 0, 0.0)); w.push_back(mk(BC_DIR_CC, 1, 0.0)); }
        }
        if (!p.yPer && !g.planar) { w.push_back(mk(BC_DIR_CC, 2, 0.0)); w.push_back(mk(BC_DIR_CC, 3, 0.0)); }
        if (p.zPer) { w.push_back(mk(BC_PER_FC, 5, 0)); w.push_back(mk(BC_PER_FC, 4, 0)); }
        else { w.push_back(mk(BC_DIR_FC, 5, 0.0)); w.push_back(mk(BC_DIR_FC, 4, 0.0)); }
    }

    // scalar.cc:185-227 (hot plate not supported; no configuration uses it)
    void initTBC() {
        std::vector<BC> &t = bcs[TF];
        t.clear();
        auto mk = [](BCType ty, int w, double v) { BC b; b.t = ty; b.wall = w; b.v = v; return b; };
        if (!p.xPer) {
            if (p.probType == 5 || p.probType == 6 || p.probType == 8) { t.push_back(mk(BC_NEU_CC, 0, 0.0)); t.push_back(mk(BC_NEU_CC, 1, 0.0)); }
            else if (p.probType == 7) { t.push_back(mk(BC_DIR_CC, 0, 1.0)); t.push_back(mk(BC_DIR_CC, 1, 0.0)); }
        }
        if (!p.yPer && !g.planar) { t.push_back(mk(BC_NEU_CC, 2, 0.0)); t.push_back(mk(BC_NEU_CC, 3, 0.0)); }
        if (p.zPer) { t.push_back(mk(BC_PER_CC, 5, 0)); t.push_back(mk(BC_PER_CC, 4, 0)); }
        else if (p.probType == 5 || p.probType == 8) { t.push_back(mk(BC_DIR_CC, 5, 0.0)); t.push_back(mk(BC_DIR_CC, 4, 1.0)); }
        else if (p.probType == 6) { t.push_back(mk(BC_DIR_CC, 5, 1.0)); t.push_back(mk(BC_DIR_CC, 4, 0.0)); }
    }

    // hydro.cc:386-461, scalar.cc:240-255
    void imposeBCs(int c) {
        Field &f = fieldOf(c);
        syncData(f.F, f, p.xPer, p.yPer, g.planar);
        for (const BC &b : bcs[c]) {
            int dim = b.wall / 2;
            if (dim == 0 && p.xPer) continue;
            if (dim == 1 && p.yPer) continue;
            imposeBC(f, b);
        }
    }

    // Metric arrays used by derivative (derivative.cc:77-105).
    const A1 &metric1(const Field &f, int d) const {
        if (d == 0) return f.stag[0] ? g.xi_xStaggr : g.xi_xColloc;
        if (d == 1) return f.stag[1] ? g.et_yStaggr : g.et_yColloc;
        return f.stag[2] ? g.zt_zStaggr : g.zt_zColloc;
    }
    const A1 &metricxx(const Field &f, int d) const {
        if (d == 0) return f.stag[0] ? g.xixxStaggr : g.xixxColloc;
        if (d == 1) return f.stag[1] ? g.etyyStaggr : g.etyyColloc;
        return f.stag[2] ? g.ztzzStaggr : g.ztzzColloc;
    }
    const A1 &metric2(const Field &f, int d) const {
        if (d == 0) return f.stag[0] ? g.xix2Staggr : g.xix2Colloc;
        if (d == 1) return f.stag[1] ? g.ety2Staggr : g.ety2Colloc;
        return f.stag[2] ? g.ztz2Staggr : g.ztz2Colloc;
    }
    double ih(int d) const { return 1.0 / (d == 0 ? g.dXi : d == 1 ? g.dEt : g.dZt); }

    // derivative::calcDerivative1_x/y/z (derivative.cc:121-164) at core points.
    double d1(const Field &f, int d, int i, int j, int k) const {
        const A3 &F = f.F;
        double fm, fp;
        if (d == 0) { fm = F(i - 1, j, k); fp = F(i + 1, j, k); }
        else if (d == 1) { fm = F(i, j - 1, k); fp = F(i, j + 1, k); }
        else { fm = F(i, j, k - 1); fp = F(i, j, k + 1); }
        double t = central12n(fm, fp);
        t *= ih(d);
        int idx = d == 0 ? i : d == 1 ? j : k;
        return metric1(f, d)(idx) * t;
    }
    // derivative::calcDerivative2xx/yy/zz (derivative.cc:178-243) at core points.
    double d2(const Field &f, int d, int i, int j, int k) const {
        const A3 &F = f.F;
        double fm, f0 = F(i, j, k), fp;
        if (d == 0) { fm = F(i - 1, j, k); fp = F(i + 1, j, k); }
        else if (d == 1) { fm = F(i, j - 1, k); fp = F(i, j + 1, k); }
        else { fm = F(i, j, k - 1); fp = F(i, j, k + 1); }
        double ihd = ih(d);
        double ih2 = std::pow(ihd, 2.0);
        double tmp = central12n(fm, fp);
        tmp *= ihd;
        double out = central22n(fm, f0, fp);
        out *= ih2;
        int idx = d == 0 ? i : d == 1 ? j : k;
        if (p.iScheme == 1) return metricxx(f, d)(idx) * tmp + 0.5 * metric2(f, d)(idx) * out;
        return metricxx(f, d)(idx) * tmp + metric2(f, d)(idx) * out;
    }

    // field.cc:309-575 interpolation slices (shift vectors) for target field tf
    // and source velocity component src (0,1,2) or temperature (3 = PcIntSlices).
    static int slices(const Field &tf, int src, int sh[4][3]) {
        bool xs = tf.stag[0], ys = tf.stag[1], zs = tf.stag[2];
        auto set = [&](int n, int a, int b, int c) { sh[n][0] = a; sh[n][1] = b; sh[n][2] = c; };
        if (!xs && ys && zs) {          // Vx
            if (src == 0) { set(0, 0, 0, 0); return 1; }
            if (src == 1) { set(0, 0, 0, 0); set(1, 0, -1, 0); set(2, 1, 0, 0); set(3, 1, -1, 0); return 4; }
            if (src == 2) { set(0, 0, 0, 0); set(1, 0, 0, -1); set(2, 1, 0, 0); set(3, 1, 0, -1); return 4; }
            set(0, 0, 0, 0); set(1, 1, 0, 0); return 2;
        }
        if (xs && !ys && zs) {          // Vy
            if (src == 0) { set(0, 0, 0, 0); set(1, -1, 0, 0); set(2, 0, 1, 0); set(3, -1, 1, 0); return 4; }
            if (src == 1) { set(0, 0, 0, 0); return 1; }
            if (src == 2) { set(0, 0, 0, 0); set(1, 0, 0, -1); set(2, 0, 1, 0); set(3, 0, 1, -1); return 4; }
            set(0, 0, 0, 0); set(1, 0, 1, 0); return 2;
        }
        if (xs && ys && !zs) {          // Vz
            if (src == 0) { set(0, 0, 0, 0); set(1, -1, 0, 0); set(2, 0, 0, 1); set(3, -1, 0, 1); return 4; }
            if (src == 1) { set(0, 0, 0, 0); set(1, 0, -1, 0); set(2, 0, 0, 1); set(3, 0, -1, 1); return 4; }
            if (src == 2) { set(0, 0, 0, 0); return 1; }
            set(0, 0, 0, 0); set(1, 0, 0, 1); return 2;
        }
        // P / T (vertex)
        if (src == 0) { set(0, 0, 0, 0); set(1, -1, 0, 0); return 2; }
        if (src == 1) { set(0, 0, 0, 0); set(1, 0, -1, 0); return 2; }
        if (src == 2) { set(0, 0, 0, 0); set(1, 0, 0, -1); return 2; }
        set(0, 0, 0, 0); return 1;
    }

    // vfield::computeDiff (vfield.cc:104-146) / sfield::computeDiff (sfield.cc:86-100)
    void computeDiff(const Field &f, A3 &H) {
        for (int d = 0; d < 3; ++d) {
            if (g.planar && d == 1) continue;   // vfield.cc:109-113, sfield.cc:91-95
#pragma omp parallel for schedule(static)
            for (int i = 0; i < f.cnt[0]; ++i) for (int j = 0; j < f.cnt[1]; ++j) for (int k = 0; k < f.cnt[2]; ++k)
                H(i, j, k) += d2(f, d, i, j, k);
        }
    }

    // vfield::computeNLin (vfield.cc:163-253) / sfield::computeNLin (sfield.cc:113-142)
    void computeNLin(const Field &f, A3 &H) {
        const Field *vsrc[3] = {&fx, &fy, &fz};
        for (int d = 0; d < 3; ++d) {
            if (g.planar && d == 1) continue;   // vfield.cc:174-190, sfield.cc:123-131
            int sh[4][3];
            int ns = slices(f, d, sh);
            const A3 &S = vsrc[d]->F;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < f.cnt[0]; ++i) for (int j = 0; j < f.cnt[1]; ++j) for (int k = 0; k < f.cnt[2]; ++k) {
                double inter = 0.0;
                for (int s = 0; s < ns; ++s) inter += S(i + sh[s][0], j + sh[s][1], k + sh[s][2]);
                double der = d1(f, d, i, j, k);
                H(i, j, k) -= inter * der / double(ns);
            }
        }
    }

    // sfield::gradient (sfield.cc:155-171) of a vertex field S into pressureGradient.
    void gradient(const A3 &S) {
        for (int i = 0; i < fx.cnt[0]; ++i) for (int j = 0; j < fx.cnt[1]; ++j) for (int k = 0; k < fx.cnt[2]; ++k)
            gradX(i, j, k) = g.xi_xColloc(i) * (S(i + 1, j, k) - S(i, j, k)) / g.dXi;
        if (!g.planar)   // sfield.cc:167-169
            for (int i = 0; i < fy.cnt[0]; ++i) for (int j = 0; j < fy.cnt[1]; ++j) for (int k = 0; k < fy.cnt[2]; ++k)
                gradY(i, j, k) = g.et_yColloc(j) * (S(i, j + 1, k) - S(i, j, k)) / g.dEt;
        for (int i = 0; i < fz.cnt[0]; ++i) for (int j = 0; j < fz.cnt[1]; ++j) for (int k = 0; k < fz.cnt[2]; ++k)
            gradZ(i, j, k) = g.zt_zColloc(k) * (S(i, j, k + 1) - S(i, j, k)) / g.dZt;
    }

    // vfield::divergence (vfield.cc:299-320)
    void divergence(A3 &divV) {
        divV.fill(0.0);
        const A3 &X = fx.F, &Y = fy.F, &Z = fz.F;
        for (int i = 0; i < fp.cnt[0]; ++i) for (int j = 0; j < fp.cnt[1]; ++j) for (int k = 0; k < fp.cnt[2]; ++k) {
            if (g.planar)   // vfield.cc:312-314
                divV(i, j, k) = g.xi_xStaggr(i) * (X(i, j, k) - X(i - 1, j, k)) / g.dXi +
                                g.zt_zStaggr(k) * (Z(i, j, k) - Z(i, j, k - 1)) / g.dZt;
            else
                divV(i, j, k) = g.xi_xStaggr(i) * (X(i, j, k) - X(i - 1, j, k)) / g.dXi +
                                g.et_yStaggr(j) * (Y(i, j, k) - Y(i, j - 1, k)) / g.dEt +
                                g.zt_zStaggr(k) * (Z(i, j, k) - Z(i, j, k - 1)) / g.dZt;
        }
    }

    // buoyantForce::addForcing (buoyantForce.cc:59-68)
    void addBuoyancy(A3 &Hz) {
        int sh[4][3];
        int ns = slices(fz, 3, sh);
        A3 inter; inter.resize(-1, -1, -1, fz.cnt[0], fz.cnt[1], fz.cnt[2]);
        for (int i = 0; i < fz.cnt[0]; ++i) for (int j = 0; j < fz.cnt[1]; ++j) for (int k = 0; k < fz.cnt[2]; ++k)
            for (int s = 0; s < ns; ++s) inter(i, j, k) += ft.F(i + sh[s][0], j + sh[s][1], k + sh[s][2]);
        for (double &x : inter.v) x /= double(ns);
        for (size_t n = 0; n < Hz.v.size(); ++n) Hz.v[n] += Fb * inter.v[n];
    }

    // Metrics of the implicit solves (hydro_d3.cc:378-400, 433-455, 488-510; scalar_d3.cc:549-571).
    void cnMetrics(int c, const A1 *&mx, const A1 *&my, const A1 *&mz) const {
        if (c == VX) { mx = &g.xix2Colloc; my = &g.ety2Staggr; mz = &g.ztz2Staggr; }
        else if (c == VY) { mx = &g.xix2Staggr; my = &g.ety2Colloc; mz = &g.ztz2Staggr; }
        else if (c == VZ) { mx = &g.xix2Staggr; my = &g.ety2Staggr; mz = &g.ztz2Colloc; }
        else { mx = &g.xix2Staggr; my = &g.ety2Staggr; mz = &g.ztz2Colloc; }   // T uses ztz2Colloc
    }

    // hydro_d3::solveVx/Vy/Vz (hydro_d3.cc:370-533), scalar_d3::solveVx..solveT (scalar_d3.cc:373-591)
    int cnSolve(int c, int *itersOut, double *errOut) {
        Field &f = fieldOf(c);
        A3 &V = f.F;
        A3 &guess = c == VX ? guessX : c == VY ? guessY : c == VZ ? guessZ : guessT;
        A3 &lapA = c == VX ? lapX : c == VY ? lapY : c == VZ ? lapZ : lapT;
        const A3 &rhs = c == VX ? nseX : c == VY ? nseY : c == VZ ? nseZ : tmpRHS;
        const A1 *mx, *my, *mz;
        cnMetrics(c, mx, my, mz);
        bool useNu = isScalar;
        double coef = (c == TF) ? kappa : nu;
        int iterCount = 0;
        double maxError = 0.0;
        while (true) {
#pragma omp parallel for schedule(static)
            for (int iX = f.blb[0]; iX <= f.bub[0]; iX++) for (int iY = f.blb[1]; iY <= f.bub[1]; iY++) for (int iZ = f.blb[2]; iZ <= f.bub[2]; iZ++) {
                if (g.planar) {   // hydro_d2.cc:293-299, scalar_d2.cc:425-431
                    double A = hz2 * (*mx)(iX) * (V(iX + 1, iY, iZ) + V(iX - 1, iY, iZ)) + hx2 * (*mz)(iZ) * (V(iX, iY, iZ + 1) + V(iX, iY, iZ - 1));
                    if (!useNu)
                        guess(iX, iY, iZ) = (A * dt / (hz2hx2 * 2.0 * p.Re) + rhs(iX, iY, iZ)) /
                                            (1.0 + dt * ((hz2 * (*mx)(iX) + hx2 * (*mz)(iZ))) / (p.Re * hz2hx2));
                    else
                        guess(iX, iY, iZ) = (A * dt * coef / (hz2hx2 * 2.0) + rhs(iX, iY, iZ)) /
                                            (1.0 + dt * coef * ((hz2 * (*mx)(iX) + hx2 * (*mz)(iZ))) / hz2hx2);
                    continue;
                }
                double A = hy2hz2 * (*mx)(iX) * (V(iX + 1, iY, iZ) + V(iX - 1, iY, iZ)) +
                           hz2hx2 * (*my)(iY) * (V(iX, iY + 1, iZ) + V(iX, iY - 1, iZ)) +
                           hx2hy2 * (*mz)(iZ) * (V(iX, iY, iZ + 1) + V(iX, iY, iZ - 1));
                double B = (hy2hz2 * (*mx)(iX) + hz2hx2 * (*my)(iY) + hx2hy2 * (*mz)(iZ));
                if (!useNu)
                    guess(iX, iY, iZ) = (A * dt / (hx2hy2hz2 * 2.0 * p.Re) + rhs(iX, iY, iZ)) /
                                        (1.0 + dt * B / (p.Re * hx2hy2hz2));
                else
                    guess(iX, iY, iZ) = (A * dt * coef / (hx2hy2hz2 * 2.0) + rhs(iX, iY, iZ)) /
                                        (1.0 + dt * coef * B / hx2hy2hz2);
            }
            V.v = guess.v;
            imposeBCs(c);
#pragma omp parallel for schedule(static)
            for (int iX = f.blb[0]; iX <= f.bub[0]; iX++) for (int iY = f.blb[1]; iY <= f.bub[1]; iY++) for (int iZ = f.blb[2]; iZ <= f.bub[2]; iZ++) {
                double L = g.planar   // hydro_d2.cc:305-309
                               ? (*mx)(iX) * (V(iX + 1, iY, iZ) - 2.0 * V(iX, iY, iZ) + V(iX - 1, iY, iZ)) / (hx2) +
                                     (*mz)(iZ) * (V(iX, iY, iZ + 1) - 2.0 * V(iX, iY, iZ) + V(iX, iY, iZ - 1)) / (hz2)
                               : (*mx)(iX) * (V(iX + 1, iY, iZ) - 2.0 * V(iX, iY, iZ) + V(iX - 1, iY, iZ)) / (hx * hx) +
                                     (*my)(iY) * (V(iX, iY + 1, iZ) - 2.0 * V(iX, iY, iZ) + V(iX, iY - 1, iZ)) / (hy * hy) +
                                     (*mz)(iZ) * (V(iX, iY, iZ + 1) - 2.0 * V(iX, iY, iZ) + V(iX, iY, iZ - 1)) / (hz * hz);
                double val = useNu ? V(iX, iY, iZ) - L * 0.5 * dt * coef
                                   : V(iX, iY, iZ) - L * 0.5 * dt * inverseRe;
                lapA(iX, iY, iZ) = std::fabs(val - rhs(iX, iY, iZ));
            }
            maxError = -INFINITY;   // blitz::max over the padded array (signed)
            for (double x : lapA.v) if (x > maxError) maxError = x;
            if (maxError < p.cnTolerance) break;
            iterCount += 1;
            if (iterCount > maxIterations) {
                if (itersOut) *itersOut = iterCount;
                if (errOut) *errOut = maxError;
                return SARAS_NOT_CONVERGED;
            }
        }
        if (itersOut) *itersOut = iterCount + 1;   // Jacobi sweeps performed
        if (errOut) *errOut = maxError;
        return SARAS_OK;
    }

    // The residual test of the loop above, for the field as it stands: max over
    // the core of |V - (nu dt / 2) L(V) - rhs| (hydro_d3.cc:392-400).
    double cnResidual(int c) {
        Field &f = fieldOf(c);
        A3 &V = f.F;
        const A3 &rhs = c == VX ? nseX : c == VY ? nseY : c == VZ ? nseZ : tmpRHS;
        const A1 *mx, *my, *mz;
        cnMetrics(c, mx, my, mz);
        const double coef = (c == TF) ? kappa : nu;
        double maxError = 0.0;
        for (int iX = f.blb[0]; iX <= f.bub[0]; iX++) for (int iY = f.blb[1]; iY <= f.bub[1]; iY++) for (int iZ = f.blb[2]; iZ <= f.bub[2]; iZ++) {
            double L = (*mx)(iX) * (V(iX + 1, iY, iZ) - 2.0 * V(iX, iY, iZ) + V(iX - 1, iY, iZ)) / (hx * hx) +
                       (*my)(iY) * (V(iX, iY + 1, iZ) - 2.0 * V(iX, iY, iZ) + V(iX, iY - 1, iZ)) / (hy * hy) +
                       (*mz)(iZ) * (V(iX, iY, iZ + 1) - 2.0 * V(iX, iY, iZ) + V(iX, iY, iZ - 1)) / (hz * hz);
            double val = isScalar ? V(iX, iY, iZ) - L * 0.5 * dt * coef : V(iX, iY, iZ) - L * 0.5 * dt * inverseRe;
            maxError = std::max(maxError, std::fabs(val - rhs(iX, iY, iZ)));
        }
        return maxError;
    }

    static void axpby(A3 &dst, double a, const A3 *src, double b) {
        if (src) for (size_t n = 0; n < dst.v.size(); ++n) dst.v[n] = a * dst.v[n] + b * src->v[n];
        else for (size_t n = 0; n < dst.v.size(); ++n) dst.v[n] = a * dst.v[n];
    }

    // hydro_d3::timeAdvance (hydro_d3.cc:254-368), scalar_d3::timeAdvance (scalar_d3.cc:243-370)
    int timeAdvance(saras_step_stats *st) {
        if (st) std::memset(st, 0, sizeof(*st));
        nseX.fill(0.0); nseY.fill(0.0); nseZ.fill(0.0);
        if (isScalar) tmpRHS.fill(0.0);
        computeDiff(fx, nseX); computeDiff(fy, nseY); computeDiff(fz, nseZ);
        double visc = isScalar ? nu : inverseRe;
        for (double &x : nseX.v) x *= visc;
        for (double &x : nseY.v) x *= visc;
        for (double &x : nseZ.v) x *= visc;
        computeNLin(fx, nseX); computeNLin(fy, nseY); computeNLin(fz, nseZ);
        if (isScalar && p.forceType == 3) addBuoyancy(nseZ);
        gradX.fill(0.0); gradY.fill(0.0); gradZ.fill(0.0);
        gradient(fp.F);
        for (size_t n = 0; n < nseX.v.size(); ++n) nseX.v[n] -= gradX.v[n];
        for (size_t n = 0; n < nseY.v.size(); ++n) nseY.v[n] -= gradY.v[n];
        for (size_t n = 0; n < nseZ.v.size(); ++n) nseZ.v[n] -= gradZ.v[n];
        for (double &x : nseX.v) x *= dt;
        for (double &x : nseY.v) x *= dt;
        for (double &x : nseZ.v) x *= dt;
        for (size_t n = 0; n < nseX.v.size(); ++n) nseX.v[n] += fx.F.v[n];
        for (size_t n = 0; n < nseY.v.size(); ++n) nseY.v[n] += fy.F.v[n];
        for (size_t n = 0; n < nseZ.v.size(); ++n) nseZ.v[n] += fz.F.v[n];
        syncData(nseX, fx, p.xPer, p.yPer, g.planar); syncData(nseY, fy, p.xPer, p.yPer, g.planar); syncData(nseZ, fz, p.xPer, p.yPer, g.planar);
        for (int c = 0; c < 3; ++c) {
            if (g.planar && c == VY) continue;   // hydro_d2.cc:242-244: solveVx, solveVz
            int it = 0; double e = 0;
            int s = cnSolve(c, &it, &e);
            if (st) st->cn_iters[c] = it;
            if (s != SARAS_OK) { if (st) st->status = s; return s; }
        }
        divergence(mgRHS);
        for (double &x : mgRHS.v) x *= 1.0 / dt;
        if (p.testPoisson) mgRHS.fill(1.0);
        long long ci0 = mg.coarseIters;
        double res = 0;
        int cyc = mg.mgSolve(Pp, mgRHS, &res);
        if (st) { st->vcycles = cyc; st->mg_residual = res; st->coarse_iters = (int)(mg.coarseIters - ci0); }
        syncData(Pp, fp, p.xPer, p.yPer, g.planar);
        if (p.testPoisson) fp.F.fill(0.0);
        for (size_t n = 0; n < fp.F.v.size(); ++n) fp.F.v[n] += Pp.v[n];
        gradient(Pp);
        for (double &x : gradX.v) x *= dt;
        for (double &x : gradY.v) x *= dt;
        for (double &x : gradZ.v) x *= dt;
        for (size_t n = 0; n < fx.F.v.size(); ++n) fx.F.v[n] -= gradX.v[n];
        for (size_t n = 0; n < fy.F.v.size(); ++n) fy.F.v[n] -= gradY.v[n];
        for (size_t n = 0; n < fz.F.v.size(); ++n) fz.F.v[n] -= gradZ.v[n];
        if (isScalar) {
            computeDiff(ft, tmpRHS);
            for (double &x : tmpRHS.v) x *= kappa;
            computeNLin(ft, tmpRHS);
            for (double &x : tmpRHS.v) x *= dt;
            for (size_t n = 0; n < tmpRHS.v.size(); ++n) tmpRHS.v[n] += ft.F.v[n];
            syncData(tmpRHS, ft, p.xPer, p.yPer, g.planar);
            int it = 0; double e = 0;
            int s = cnSolve(TF, &it, &e);
            if (st) st->cn_iters[3] = it;
            if (s != SARAS_OK) { if (st) st->status = s; return s; }
        }
        imposeBCs(VX);
        if (!g.planar) imposeBCs(VY);   // hydro_d2.cc:278-279: imposeUBCs, imposeWBCs
        imposeBCs(VZ);
        if (isScalar) imposeBCs(TF);
        return SARAS_OK;
    }

    // tseries::writeTSData (tseries.cc:137-178, 195-246) at np = 1.
    // field::fieldMax (field.cc:602-617): max |F| over the padded array.
    static double fieldMax(const A3 &F) {
        double m = 0.0;
        for (double x : F.v) m = std::max(m, std::fabs(x));
        return m;
    }

    // vfield::computeTStp (vfield.cc:267-284).
    void computeTStp(double &dtOut) const {
        double delx = g.dXi, dely = g.dEt, delz = g.dZt;
        double Umax = fieldMax(fx.F), Vmax = fieldMax(fy.F), Wmax = fieldMax(fz.F);
        if (g.planar) { dely = 0.0; Vmax = 1.0; }   // vfield.cc:273-279
        dtOut = p.courantNumber * (delx / Umax + dely / Vmax + delz / Wmax);
    }

    int diagnostics(double *energy, double *maxDiv, double *nusselt) {
        A3 divV; divV.resize(-1, -1, -1, fp.cnt[0], fp.cnt[1], fp.cnt[2]);
        divergence(divV);
        double md = -INFINITY;   // fxMax over the collocated core range
        for (int i = 0; i < g.collocCoreSize[0]; ++i) for (int j = 0; j < g.collocCoreSize[1]; ++j) for (int k = 0; k < g.collocCoreSize[2]; ++k)
            md = std::max(md, divV(i, j, k));
        double localEnergy = 0.0, localUzT = 0.0;
        for (int iX = 0; iX <= fp.cnt[0] - 1; iX++) for (int iY = 0; iY <= fp.cnt[1] - 1; iY++) for (int iZ = 0; iZ <= fp.cnt[2] - 1; iZ++) {
            double dv = (g.dXi / g.xi_xColloc(iX)) * (g.dEt / g.et_yColloc(iY)) * (g.dZt / g.zt_zColloc(iZ));
            if (g.planar) {   // tseries.cc:149-156, 210-219
                localEnergy += (std::pow((fx.F(iX - 1, iY, iZ) + fx.F(iX, iY, iZ)) / 2.0, 2.0) +
                                std::pow((fz.F(iX, iY, iZ - 1) + fz.F(iX, iY, iZ)) / 2.0, 2.0)) *
                               (g.dXi / g.xi_xColloc(iX)) * (g.dZt / g.zt_zColloc(iZ));
                if (isScalar)
                    localUzT += ((fz.F(iX, iY, iZ) + fz.F(iX, iY, iZ - 1)) / 2.0) * ft.F(iX, iY, iZ) * (g.dXi / g.xi_xColloc(iX)) *
                                (g.dZt / g.zt_zColloc(iZ));
                continue;
            }
            localEnergy += (std::pow((fx.F(iX - 1, iY, iZ) + fx.F(iX, iY, iZ)) / 2.0, 2.0) +
                            std::pow((fy.F(iX, iY - 1, iZ) + fy.F(iX, iY, iZ)) / 2.0, 2.0) +
                            std::pow((fz.F(iX, iY, iZ - 1) + fz.F(iX, iY, iZ)) / 2.0, 2.0)) *
                           (g.dXi / g.xi_xColloc(iX)) * (g.dEt / g.et_yColloc(iY)) * (g.dZt / g.zt_zColloc(iZ));
            if (isScalar)
                localUzT += ((fz.F(iX, iY, iZ) + fz.F(iX, iY, iZ - 1)) / 2.0) * ft.F(iX, iY, iZ) *
                            (g.dXi / g.xi_xColloc(iX)) * (g.dEt / g.et_yColloc(iY)) * (g.dZt / g.zt_zColloc(iZ));
            (void)dv;
        }
        if (energy) *energy = localEnergy / totalVol;
        if (maxDiv) *maxDiv = md;
        if (nusselt) *nusselt = isScalar ? 1.0 + (localUzT / totalVol) / kappa : 0.0;
        return md > 1.0e5 ? SARAS_DIVERGENCE_LIMIT : SARAS_OK;
    }

    // hydro_d3::testPeriodic (hydro_d3.cc:536-679)
    double hydroTestPeriodic() {
        const double PI = M_PI;
        nseX.fill(0); nseY.fill(0); nseZ.fill(0);
        fx.F.fill(0); fy.F.fill(0); fz.F.fill(0);
        for (int i = -1; i <= fx.cnt[0]; i++) for (int j = -1; j <= fx.cnt[1]; j++) for (int k = -1; k <= fx.cnt[2]; k++) {
            fx.F(i, j, k) = std::sin(2.0 * PI * g.xColloc(i) / g.xLen) * std::cos(2.0 * PI * g.yStaggr(j) / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
            nseX(i, j, k) = fx.F(i, j, k);
        }
        for (int i = -1; i <= fy.cnt[0]; i++) for (int j = -1; j <= fy.cnt[1]; j++) for (int k = -1; k <= fy.cnt[2]; k++) {
            fy.F(i, j, k) = -std::cos(2.0 * PI * g.xStaggr(i) / g.xLen) * std::sin(2.0 * PI * g.yColloc(j) / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
            nseY(i, j, k) = fy.F(i, j, k);
        }
        // Expected pad values (pad width 1): the analytic function at the mirrored coordinate.
        {
            int lo = 0, hi = fx.cnt[0] - 1;
            double xl = g.xColloc(lo) - (g.xColloc(lo + 1) - g.xColloc(lo)), xh = g.xColloc(hi) + (g.xColloc(hi) - g.xColloc(hi - 1));
            for (int j = 0; j < fx.cnt[1]; j++) for (int k = 0; k < fx.cnt[2]; k++) {
                nseX(lo - 1, j, k) = std::sin(2.0 * PI * xl / g.xLen) * std::cos(2.0 * PI * g.yStaggr(j) / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
                nseX(hi + 1, j, k) = std::sin(2.0 * PI * xh / g.xLen) * std::cos(2.0 * PI * g.yStaggr(j) / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
            }
            lo = 0; hi = fx.cnt[1] - 1;
            double yl = g.yStaggr(lo) - (g.yStaggr(lo + 1) - g.yStaggr(lo)), yh = g.yStaggr(hi) + (g.yStaggr(hi) - g.yStaggr(hi - 1));
            for (int i = 0; i < fx.cnt[0]; i++) for (int k = 0; k < fx.cnt[2]; k++) {
                nseX(i, lo - 1, k) = std::sin(2.0 * PI * g.xColloc(i) / g.xLen) * std::cos(2.0 * PI * yl / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
                nseX(i, hi + 1, k) = std::sin(2.0 * PI * g.xColloc(i) / g.xLen) * std::cos(2.0 * PI * yh / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
            }
            lo = 0; hi = fx.cnt[2] - 1;
            double zl = g.zStaggr(lo) - (g.zStaggr(lo + 1) - g.zStaggr(lo)), zh = g.zStaggr(hi) + (g.zStaggr(hi) - g.zStaggr(hi - 1));
            for (int i = 0; i < fx.cnt[0]; i++) for (int j = 0; j < fx.cnt[1]; j++) {
                nseX(i, j, lo - 1) = std::sin(2.0 * PI * g.xColloc(i) / g.xLen) * std::cos(2.0 * PI * g.yStaggr(j) / g.yLen) * std::cos(2.0 * PI * zl / g.zLen);
                nseX(i, j, hi + 1) = std::sin(2.0 * PI * g.xColloc(i) / g.xLen) * std::cos(2.0 * PI * g.yStaggr(j) / g.yLen) * std::cos(2.0 * PI * zh / g.zLen);
            }
        }
        {
            int lo = 0, hi = fy.cnt[0] - 1;
            double xl = g.xStaggr(lo) - (g.xStaggr(lo + 1) - g.xStaggr(lo)), xh = g.xStaggr(hi) + (g.xStaggr(hi) - g.xStaggr(hi - 1));
            for (int j = 0; j < fy.cnt[1]; j++) for (int k = 0; k < fy.cnt[2]; k++) {
                nseY(lo - 1, j, k) = -std::cos(2.0 * PI * xl / g.xLen) * std::sin(2.0 * PI * g.yColloc(j) / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
                nseY(hi + 1, j, k) = -std::cos(2.0 * PI * xh / g.xLen) * std::sin(2.0 * PI * g.yColloc(j) / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
            }
            lo = 0; hi = fy.cnt[1] - 1;
            double yl = g.yColloc(lo) - (g.yColloc(lo + 1) - g.yColloc(lo)), yh = g.yColloc(hi) + (g.yColloc(hi) - g.yColloc(hi - 1));
            for (int i = 0; i < fy.cnt[0]; i++) for (int k = 0; k < fy.cnt[2]; k++) {
                nseY(i, lo - 1, k) = -std::cos(2.0 * PI * g.xStaggr(i) / g.xLen) * std::sin(2.0 * PI * yl / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
                nseY(i, hi + 1, k) = -std::cos(2.0 * PI * g.xStaggr(i) / g.xLen) * std::sin(2.0 * PI * yh / g.yLen) * std::cos(2.0 * PI * g.zStaggr(k) / g.zLen);
            }
            lo = 0; hi = fy.cnt[2] - 1;
            double zl = g.zStaggr(lo) - (g.zStaggr(lo + 1) - g.zStaggr(lo)), zh = g.zStaggr(hi) + (g.zStaggr(hi) - g.zStaggr(hi - 1));
            for (int i = 0; i < fy.cnt[0]; i++) for (int j = 0; j < fy.cnt[1]; j++) {
                nseY(i, j, lo - 1) = -std::cos(2.0 * PI * g.xStaggr(i) / g.xLen) * std::sin(2.0 * PI * g.yColloc(j) / g.yLen) * std::cos(2.0 * PI * zl / g.zLen);
                nseY(i, j, hi + 1) = -std::cos(2.0 * PI * g.xStaggr(i) / g.xLen) * std::sin(2.0 * PI * g.yColloc(j) / g.yLen) * std::cos(2.0 * PI * zh / g.zLen);
            }
        }
        imposeBCs(VX); imposeBCs(VY); imposeBCs(VZ);
        // V -= nseRHS, max over the faces (corner/edge pads of the expected
        // arrays keep the initial analytic values and are compared too).
        double m = 0.0;
        for (size_t n = 0; n < fx.F.v.size(); ++n) m = std::max(m, std::fabs(fx.F.v[n] - nseX.v[n]));
        for (size_t n = 0; n < fy.F.v.size(); ++n) m = std::max(m, std::fabs(fy.F.v[n] - nseY.v[n]));
        return m;
    }
};

struct Handle {
    Solver s;
};

A3 *fieldArray(Solver &s, int id) {
    switch (id) {
    case SARAS_FIELD_VX: return &s.fx.F;
    case SARAS_FIELD_VY: return &s.fy.F;
    case SARAS_FIELD_VZ: return &s.fz.F;
    case SARAS_FIELD_P: return &s.fp.F;
    case SARAS_FIELD_T: return &s.ft.F;
    case SARAS_FIELD_PP: return &s.Pp;
    case SARAS_FIELD_MGRHS: return &s.mgRHS;
    case SARAS_FIELD_NSE_X: return &s.nseX;
    case SARAS_FIELD_NSE_Y: return &s.nseY;
    case SARAS_FIELD_NSE_Z: return &s.nseZ;
    case SARAS_FIELD_TRHS: return &s.tmpRHS;
    case SARAS_FIELD_GRAD_X: return &s.gradX;
    case SARAS_FIELD_GRAD_Y: return &s.gradY;
    case SARAS_FIELD_GRAD_Z: return &s.gradZ;
    }
    return nullptr;
}

}  // namespace

// ------------------------------------------------------------------ C API
extern "C" {

void *orc_create(const saras_params *p) {
    Handle *h = new Handle();
    h->s.build(*p);
    return h;
}
void orc_destroy(void *h) { delete (Handle *)h; }

int orc_field_dims(void *h, int field, int *dims) {
    A3 *a = fieldArray(((Handle *)h)->s, field);
    if (!a) return SARAS_BAD_ARG;
    for (int d = 0; d < 3; ++d) dims[d] = (int)a->n[d];
    return SARAS_OK;
}
int orc_get(void *h, int field, double *out) {
    A3 *a = fieldArray(((Handle *)h)->s, field);
    if (!a) return SARAS_BAD_ARG;
    std::memcpy(out, a->v.data(), a->v.size() * sizeof(double));
    return SARAS_OK;
}
int orc_set(void *h, int field, const double *in) {
    A3 *a = fieldArray(((Handle *)h)->s, field);
    if (!a) return SARAS_BAD_ARG;
    std::memcpy(a->v.data(), in, a->v.size() * sizeof(double));
    return SARAS_OK;
}
int orc_apply_bc(void *h, int field) {
    Solver &s = ((Handle *)h)->s;
    int c = field == SARAS_FIELD_VX ? VX : field == SARAS_FIELD_VY ? VY : field == SARAS_FIELD_VZ ? VZ : field == SARAS_FIELD_T ? TF : -1;
    if (c < 0) return SARAS_BAD_ARG;
    s.imposeBCs(c);
    return SARAS_OK;
}
int orc_sync_field(void *h, int field) {
    Solver &s = ((Handle *)h)->s;
    A3 *a = fieldArray(s, field);
    if (!a) return SARAS_BAD_ARG;
    const Field *f = (field == SARAS_FIELD_VX || field == SARAS_FIELD_NSE_X || field == SARAS_FIELD_GRAD_X) ? &s.fx :
                     (field == SARAS_FIELD_VY || field == SARAS_FIELD_NSE_Y || field == SARAS_FIELD_GRAD_Y) ? &s.fy :
                     (field == SARAS_FIELD_VZ || field == SARAS_FIELD_NSE_Z || field == SARAS_FIELD_GRAD_Z) ? &s.fz : &s.fp;
    syncData(*a, *f, s.p.xPer, s.p.yPer, s.g.planar);
    return SARAS_OK;
}
int orc_vfield_compute_diff(void *h) {
    Solver &s = ((Handle *)h)->s;
    s.computeDiff(s.fx, s.nseX); s.computeDiff(s.fy, s.nseY); s.computeDiff(s.fz, s.nseZ);
    return SARAS_OK;
}
int orc_vfield_compute_nlin(void *h) {
    Solver &s = ((Handle *)h)->s;
    s.computeNLin(s.fx, s.nseX); s.computeNLin(s.fy, s.nseY); s.computeNLin(s.fz, s.nseZ);
    return SARAS_OK;
}
int orc_sfield_gradient(void *h, int sf) {
    Solver &s = ((Handle *)h)->s;
    A3 *a = fieldArray(s, sf);
    if (!a) return SARAS_BAD_ARG;
    s.gradient(*a);
    return SARAS_OK;
}
int orc_vfield_divergence(void *h) {
    Solver &s = ((Handle *)h)->s;
    s.divergence(s.mgRHS);
    return SARAS_OK;
}
int orc_tfield_compute_diff(void *h) { Solver &s = ((Handle *)h)->s; s.computeDiff(s.ft, s.tmpRHS); return SARAS_OK; }
int orc_tfield_compute_nlin(void *h) { Solver &s = ((Handle *)h)->s; s.computeNLin(s.ft, s.tmpRHS); return SARAS_OK; }
int orc_axpby(void *h, int dst, double a, int src, double b) {
    Solver &s = ((Handle *)h)->s;
    A3 *D = fieldArray(s, dst);
    A3 *S = src >= 0 ? fieldArray(s, src) : nullptr;
    if (!D || (src >= 0 && (!S || S->v.size() != D->v.size()))) return SARAS_BAD_ARG;
    Solver::axpby(*D, a, S, b);
    return SARAS_OK;
}
int orc_cn_solve(void *h, int comp, int *iters, double *err) {
    Solver &s = ((Handle *)h)->s;
    int c = comp == 3 ? TF : comp;
    return s.cnSolve(c, iters, err);
}
int orc_mg_solve(void *h, int *cycles, double *res) {
    Solver &s = ((Handle *)h)->s;
    long long c0 = s.mg.coarseIters;
    int c = s.mg.mgSolve(s.Pp, s.mgRHS, res);
    (void)c0;
    if (cycles) *cycles = c;
    return SARAS_OK;
}
long long orc_coarse_iters(void *h) { return ((Handle *)h)->s.mg.coarseIters; }
int orc_time_advance(void *h, saras_step_stats *st) { return ((Handle *)h)->s.timeAdvance(st); }
int orc_cn_residual(void *h, int comp, double *res) {
    if (comp < 0 || comp > 3) return SARAS_BAD_ARG;
    *res = ((Handle *)h)->s.cnResidual(comp == 3 ? TF : comp);
    return SARAS_OK;
}
int orc_diagnostics(void *h, double *e, double *d, double *nu) { return ((Handle *)h)->s.diagnostics(e, d, nu); }
int orc_compute_tstp(void *h, double *dt) { ((Handle *)h)->s.computeTStp(*dt); return SARAS_OK; }
int orc_set_dt(void *h, double dt) { ((Handle *)h)->s.dt = dt; return SARAS_OK; }
int orc_mg_test_prolong(void *h, double *err) { *err = ((Handle *)h)->s.mg.testProlong(); return SARAS_OK; }
int orc_mg_test_transfer(void *h, double *err) { *err = ((Handle *)h)->s.mg.testTransfer(); return SARAS_OK; }
int orc_mg_test_periodic(void *h, double *err) { *err = ((Handle *)h)->s.mg.testPeriodic(); return SARAS_OK; }
int orc_hydro_test_periodic(void *h, double *err) { *err = ((Handle *)h)->s.hydroTestPeriodic(); return SARAS_OK; }

int orc_mg_level_dims(void *h, int level, int *dims) {
    Multigrid &m = ((Handle *)h)->s.mg;
    if (level < 0 || level > m.d) return SARAS_BAD_ARG;
    dims[0] = m.xEnd[level] + 3; dims[1] = m.yEnd[level] + 3; dims[2] = m.zEnd[level] + 3;
    return SARAS_OK;
}
int orc_mg_set_level(void *h, int level, int which, const double *in) {
    Multigrid &m = ((Handle *)h)->s.mg;
    if (level < 0 || level > m.d) return SARAS_BAD_ARG;
    A3 &a = which == 0 ? m.pressureData[level] : m.residualData[level];
    std::memcpy(a.v.data(), in, a.v.size() * sizeof(double));
    return SARAS_OK;
}
int orc_mg_get_level(void *h, int level, int which, double *out) {
    Multigrid &m = ((Handle *)h)->s.mg;
    if (level < 0 || level > m.d) return SARAS_BAD_ARG;
    A3 &a = which == 0 ? m.pressureData[level] : m.residualData[level];
    std::memcpy(out, a.v.data(), a.v.size() * sizeof(double));
    return SARAS_OK;
}
int orc_mg_smooth(void *h, int level, int count) {
    Multigrid &m = ((Handle *)h)->s.mg;
    if (level < 0 || level > m.d) return SARAS_BAD_ARG;
    m.vLevel = level; m.zeroBC = (level != 0);
    if (level == m.d && count < 0) m.solve(); else m.smooth(count);
    return SARAS_OK;
}
int orc_mg_restrict(void *h, int level) {
    Multigrid &m = ((Handle *)h)->s.mg;
    if (level < 0 || level >= m.d) return SARAS_BAD_ARG;
    m.vLevel = level;
    m.computeResidual();
    m.coarsen();
    return SARAS_OK;
}
int orc_mg_prolong_add(void *h, int level) {
    Multigrid &m = ((Handle *)h)->s.mg;
    if (level < 0 || level >= m.d) return SARAS_BAD_ARG;
    m.smoothedPres[level] = m.pressureData[level];
    m.vLevel = level + 1;
    m.prolong();
    A3 &P = m.pressureData[level];
    for (size_t n = 0; n < P.v.size(); ++n) P.v[n] += m.smoothedPres[level].v[n];
    return SARAS_OK;
}
int orc_mg_compute_error(void *h, int norm, double *err) {
    Multigrid &m = ((Handle *)h)->s.mg;
    m.vLevel = 0;
    *err = m.computeError(norm);
    return SARAS_OK;
}

}  // extern "C"
