// context.cuh -- the solver context behind the C ABI.
#pragma once

#include <cuda.h>

#include "common.cuh"

struct saras_ctx;

namespace saras {

// Kernels with CUDA-event timing (saras_profile_*).
enum ProfKernel : int {
    PK_MG_SMOOTH64 = 0,   // FP64 Jacobi sweep, level 0
    PK_MG_SMOOTH32,       // FP32 Jacobi sweep, level 0 (mixed mode)
    PK_MG_RESID64,        // FP64 residual (+restriction input), level 0
    PK_MG_RESID32,
    PK_MG_RESTRICT64,
    PK_MG_RESTRICT32,
    PK_MG_PROLONG64,
    PK_MG_PROLONG32,
    PK_REFINE_RESID,      // FP64 fine residual + FP32 demotion (mixed)
    PK_REFINE_UPDATE,     // FP64 correction accumulation (mixed)
    PK_RHS,               // fused NSE right-hand side
    PK_CN,                // fused CN Jacobi sweep + BC + residual
    PK_PROJECT,
    PK_DIVERGENCE,
    PK_CONV_FWD,          // U-Net implicit-GEMM convolution (tcgen05)
    PK_CONV_BWD,
    PK_GUESS,             // initial guess of a target-mode solve: histories, restrictions, network, guess
    PK_COUNT
};

struct ProfSlot {
    bool enabled = false;
    std::vector<cudaEvent_t> ev;   // start/stop pairs
    long long launches = 0;
    double bytes = 0.0;
    double ms = 0.0;
};

// A profiling event recorded while a V-cycle was captured as a CUDA graph: an
// event-record node of the graph, which every replay points at a fresh event.
struct ProfNode {
    cudaEvent_t captured = nullptr;   // the event recorded at capture time
    cudaGraphNode_t node = nullptr;
    int slot = 0;
    bool end = false;                 // stop event (closes one launch of the slot)
    double bytes = 0.0;
};

// One multigrid level in both precisions.
struct Level {
    int n[3];                 // core index range 0..n (n = 2^(ind-l)), padded n+3
    long count;               // padded point count
    double *a = nullptr, *b = nullptr, *r = nullptr;   // FP64 pressure ping-pong + rhs
    int cur = 0;              // 0: a holds pressureData, 1: b
    float *a32 = nullptr, *b32 = nullptr, *r32 = nullptr;
    int cur32 = 0;
    double hx, hy, hz, hxhy, hyhz, hzhx, hxhyhz;
    // uniform-grid stencil coefficients (exact products of the reference expressions)
    double cx, cy, cz, c7, den;      // smoother: hyhz*xix2, hzhx*ety2, hxhy*ztz2, 2*hxhyhz, 4*(...)
    double lx, ly, lz;               // residual: xix2/(hx*hx) folded as products with 1/(hx*hx)
    double ihx2, ihy2, ihz2;         // 1/(hx*hx) (exact powers of two)
    // stretched meshes: the level's staggered metrics xix2, xixx, ety2, etyy,
    // ztz2, ztzz (poisson.cc:463-495), device pointers at index 0
    double *metBlock = nullptr;
    double hx2 = 0, hz2 = 0;         // 2D: pow(2^l dXi, 2), pow(2^l dZt, 2) (poisson.cc:426-428)
    int planar = 0;
    const double *xix2 = nullptr, *xixx = nullptr, *ety2 = nullptr, *etyy = nullptr, *ztz2 = nullptr, *ztzz = nullptr;
    double *pa() const { return cur == 0 ? a : b; }
    double *pb() const { return cur == 0 ? b : a; }
    float *pa32() const { return cur32 == 0 ? a32 : b32; }
    float *pb32() const { return cur32 == 0 ? b32 : a32; }
};

// Per-field metadata: core counts, staggering, bulk box, boundary programs.
struct FieldInfo {
    int n[3] = {0, 0, 0};
    bool stag[3] = {false, false, false};
    int blo[3], bhi[3];
    BcProgram full;      // syncData + wall objects (imposeXBCs)
    BcProgram sync;      // syncData alone
};

struct Ctx {
    saras_params p;
    int dev = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copyStream[SARAS_NUM_FIELDS] = {};   // saras_upload_fields / saras_download_fields
    cudaEvent_t copyEvent[SARAS_NUM_FIELDS + 1] = {};
    bool scalar = false;
    // grid (grid.cc:59-136)
    int Ns[3], Nc[3];
    double dXi[3], ih[3], ih2[3], L[3];
    double m1[3], m2[3];           // uniform metrics xi_x (=1/L) and xix2 (=pow(1/L,2))
    // Coordinates and metrics of every axis d at the collocated (s = 0) and the
    // staggered (s = 1) points, kind 0 xi_x, 1 xixx, 2 xix2 (grid.cc:290-320,
    // 370-422, 442-519): uniform values everywhere, the tangent-hyperbolic map
    // on the core of a stretched axis.  Host arrays start at index -1; device
    // pointers point at index 0.
    bool stretched = false;        // some axis has Mesh Type 'D'
    // the 2D (PLANAR) solver: "Y Index" 0, one y point (grid.cc:88-92, 232-234);
    // every y term of the stencils is left out and Vy takes no part
    bool planar = false;
    std::vector<double> hmet[3][2][3], hcoord[3][2];
    double *dmet = nullptr;
    const double *met[3][2][3] = {};
    double inverseRe, nu, kappa, Fb, dt;
    double hx2hy2, hy2hz2, hz2hx2, hx2hy2hz2;
    int maxIterations;
    double totalVol;
    // fields
    FieldInfo info[SARAS_NUM_FIELDS];
    double *f[SARAS_NUM_FIELDS] = {nullptr};
    double *scratch[4] = {nullptr, nullptr, nullptr, nullptr};   // ping-pong partners of Vx, Vy, Vz, T
    // multigrid
    std::vector<Level> lv;
    int depth = 0;
    int mgMode = SARAS_MG_REFERENCE;
    double mgTarget = 1e-8;
    int mgMaxCycles = 200;
    int maxCount = 0;
    int numSMs = 1;           // multiprocessors of the context's device
    // finest-level FP32 plane-streaming stencils (TMA, target modes): tensor
    // maps of the two iterate buffers (a32, b32) with the main and the side
    // box and of the right-hand side (r32), and the launch shape; planeOk
    // false when the level does not fit
    bool planeOk = false;
    CUtensorMap planeMap[2], planeSide[2], planeR;
    int planeMainRows = 0, planeSideRows = 0, planeRRows = 0, planeSideOff = 0, planeROff = 0, planeSlotFloats = 0, planeSegPlanes = 0,
        planeSegs = 0, planeMaxQ = 0;
    size_t planeSmem = 0;
    double *wallX = nullptr, *wallY = nullptr, *wallZ = nullptr;   // Dirichlet check walls
    // reductions
    double *red = nullptr;          // partial sums (device)
    int redCap = 0;
    double *dscal = nullptr;        // device scalars
    void *probeBuf = nullptr;       // probe indices and values (grown on demand)
    size_t probeBytes = 0;
    double *hscal = nullptr;        // pinned host mirror
    int *dflag = nullptr;
    // stats
    long long launches = 0;
    long long coarseIters = 0;
    saras_step_stats last{};
    // learned warm start
    int guessMode = SARAS_GUESS_PREVIOUS;
    void *unet = nullptr;
    double *pHist[3] = {nullptr, nullptr, nullptr};   // Pp of the three previous steps (newest first)
    long long *fx[3] = {nullptr, nullptr, nullptr};   // level-0 fixed-point iterate ping-pong + rhs (mixed mode)
    float *cnp = nullptr;      // split-FP64 Jacobi solve: N0 of each component and the D ping-pong (float pairs)
    long cnpCount = 0;
    int n0Fresh[4] = {0, 0, 0, 0};   // N0 of component q written by this step's right-hand side
    int cnSweeps[4] = {2, 2, 2, 2};  // split Jacobi sweeps the last solve of component q launched
    int tailLt = -1;          // first level of the fused coarse V-cycle tail (target modes), or -1
    double rhoMixed = 0.1;    // measured residual contraction per FP32 V-cycle (mixed mode, mixedCycles = 0)
    int coarseN = 0;          // coarsest core points solved by coarseM (0: Gauss-Seidel instead)
    double *coarseM64 = nullptr;   // coarsest-level solution operator (coarseN x coarseN, row-major)
    float *coarseM32 = nullptr;
    // target-mode V-cycles replayed as CUDA graphs: [FP32?][zero start?]
    // [FP32?][zero start?][timed?]: with profiling on, the timed instance holds
    // the profiling event nodes and replays one cycle in profEvery
    cudaGraphExec_t vgraph[2][2][2] = {};
    cudaGraph_t vgraphSrc[2][2][2] = {};      // kept for the event-node handles
    std::vector<ProfNode> vgraphProf[2][2][2];   // profiling event nodes of each graph, in capture order
    bool profCapturing = false;               // prof_begin / prof_end record graph event nodes
    bool profSuppress = false;                // prof_begin / prof_end record nothing (untimed capture)
    int profEvery = 1;
    long long profReplays = 0;
    std::vector<ProfNode> profCaptured;
    long long vgraphLaunches[2][2][2] = {};
    std::vector<int> vgraphState[2][2][2];
    int histCount = 0;
    bool ppInHist = false;    // Pp's buffer moved to pHist[0] by unet_begin_solve; the solve has not written Pp yet
    bool collecting = false;
    // profiling
    ProfSlot prof[PK_COUNT];
    std::vector<cudaEvent_t> evPool;          // timing events not in use
    cudaEvent_t userEv[16] = {nullptr};
    std::string err;
};

// ---- launch accounting and profiling (host side)
void prof_begin(Ctx &c, int k, int level);
void prof_end(Ctx &c, int k, int level, double bytes);
inline void count_launch(Ctx &c, int n = 1) { c.launches += n; }

// ---- field operations (fields.cu)
int fields_setup(Ctx &c);
int apply_bc(Ctx &c, int field);
int sync_field(Ctx &c, int field);
int vfield_compute_diff(Ctx &c);
int vfield_compute_nlin(Ctx &c);
int sfield_gradient(Ctx &c, int sf);
int vfield_divergence(Ctx &c, double *dst, bool scale_dt);
int tfield_compute_diff(Ctx &c);
int tfield_compute_nlin(Ctx &c);
int axpby(Ctx &c, int dst, double a, int src, double b);
int compute_rhs(Ctx &c);
int compute_trhs(Ctx &c);
int cn_solve(Ctx &c, int comp, int *iters, double *maxerr);
int project(Ctx &c, bool with_bc);
int diagnostics(Ctx &c, double *energy, double *maxdiv, double *nusselt);
int compute_tstp(Ctx &c, double *dt);
int probe(Ctx &c, int n, const int *ijk, int nf, const int *fields, double *out);
int hydro_test_periodic(Ctx &c, double *err);
int time_advance(Ctx &c, saras_step_stats *st);

// ---- multigrid (multigrid.cu)
int mg_setup(Ctx &c);
void mg_free(Ctx &c);
int mg_solve(Ctx &c, int *cycles, double *residual, saras_step_stats *st);
int mg_smooth_level(Ctx &c, int level, int count);
int mg_restrict_level(Ctx &c, int level);
int mg_prolong_level(Ctx &c, int level);
int mg_compute_error(Ctx &c, int norm, double *err);
int mg_set_level(Ctx &c, int level, int which, const double *host);
int mg_get_level(Ctx &c, int level, int which, double *host);
int mg_test_prolong(Ctx &c, double *err);
int mg_test_transfer(Ctx &c, double *err);
int mg_test_periodic(Ctx &c, double *err);

// ---- learned warm start (unet.cu)
int unet_create(Ctx &c);
void unet_free(Ctx &c);
int unet_collect(Ctx &c);
int unet_train(Ctx &c, int iters, double lr, double *loss);
int unet_infer(Ctx &c, double *out);
int unet_shape(Ctx &c, long long *nparam, int dims[3]);
int unet_grad_check(Ctx &c, const float *feat, const float *target, const float *params, float *out, double *loss, float *grad);
int unet_begin_solve(Ctx &c);
int unet_guess(Ctx &c, const double *b, double *dst, int mode, long long *fxdst = nullptr, int sc = 0, int *flag = nullptr);
void vgraph_reset(Ctx &c);
int prof_graph_replay(Ctx &c, cudaGraphExec_t ge, const std::vector<ProfNode> &nodes);
int unet_pick(Ctx &c);
bool unet_tracking(const Ctx &c);
int unet_shadow(Ctx &c, int built);
void unet_note_start(Ctx &c, int built, double rel);
int unet_collect_sample(Ctx &c, const double *b);
int conv3d_check(int mode, int D, int H, int W, int cin, int cout, const unsigned short *x, const unsigned short *dy,
                 const float *w, const float *bias, int relu, float *out);

// ---- reductions (fields.cu)
int reduce_sum_partials(Ctx &c, int nparts, double *host_out);

}  // namespace saras

struct saras_ctx {
    saras::Ctx c;
};
