// capi.cu -- the extern "C" entry points of include/saras_gb300.h, the
// parameters.yaml reader and the per-kernel CUDA-event profiler.

#include <cmath>
#include <cstring>
#include <cctype>
#include <fstream>
#include <sstream>
#include <string>
#include <map>
#include <algorithm>
#include <array>
#include <cstdio>
#include <vector>

#include "context.cuh"

namespace saras {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }

// ------------------------------------------------------------------ profiler
// While a V-cycle is being captured as a CUDA graph the events are recorded as
// external event-record nodes of the graph (cudaEventRecordExternal), and
// prof_graph_replay gives those nodes fresh events at every replay, so the
// slots keep timing their kernels inside replayed graphs.
static void prof_capture_event(Ctx &c, int k, bool end, double bytes) {
    ProfNode n;
    cudaEventCreate(&n.captured);
    cudaEventRecordWithFlags(n.captured, c.stream, cudaEventRecordExternal);
    n.slot = k;
    n.end = end;
    n.bytes = bytes;
    c.profCaptured.push_back(n);
}

// Timing events come from a pool (created once, returned by prof_drain), so
// profiling a replayed V-cycle costs its event-node updates and no event
// creation on the host path between the GPU's launches.
static cudaEvent_t prof_event(Ctx &c) {
    if (!c.evPool.empty()) {
        cudaEvent_t e = c.evPool.back();
        c.evPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

void prof_begin(Ctx &c, int k, int level) {
    if (level != 0 || k < 0 || k >= PK_COUNT || !c.prof[k].enabled || c.profSuppress) return;
    if (c.profCapturing) { prof_capture_event(c, k, false, 0.0); return; }
    cudaEvent_t e = prof_event(c);
    cudaEventRecord(e, c.stream);
    c.prof[k].ev.push_back(e);
}

static void prof_drain(Ctx &c, int k) {
    ProfSlot &s = c.prof[k];
    if (s.ev.size() < 2) return;
    cudaEventSynchronize(s.ev.back());
    size_t pairs = s.ev.size() / 2;
    for (size_t q = 0; q < pairs; ++q) {
        float ms = 0;
        cudaEventElapsedTime(&ms, s.ev[2 * q], s.ev[2 * q + 1]);
        s.ms += ms;
        c.evPool.push_back(s.ev[2 * q]);
        c.evPool.push_back(s.ev[2 * q + 1]);
    }
    s.ev.erase(s.ev.begin(), s.ev.begin() + 2 * pairs);
}

void prof_end(Ctx &c, int k, int level, double bytes) {
    if (level != 0 || k < 0 || k >= PK_COUNT || !c.prof[k].enabled || c.profSuppress) return;
    if (c.profCapturing) { prof_capture_event(c, k, true, bytes); return; }
    cudaEvent_t e = prof_event(c);
    cudaEventRecord(e, c.stream);
    c.prof[k].ev.push_back(e);
    c.prof[k].launches += 1;
    c.prof[k].bytes += bytes;
    if (c.prof[k].ev.size() >= 8192) prof_drain(c, k);
}

int prof_graph_replay(Ctx &c, cudaGraphExec_t ge, const std::vector<ProfNode> &nodes) {
    for (const ProfNode &n : nodes) {
        cudaEvent_t e = prof_event(c);
        if (!e) return SARAS_CUDA_ERROR;
        if (cudaGraphExecEventRecordNodeSetEvent(ge, n.node, e) != cudaSuccess) {
            c.evPool.push_back(e);
            return SARAS_CUDA_ERROR;
        }
        ProfSlot &s = c.prof[n.slot];
        s.ev.push_back(e);
        if (n.end) { s.launches += 1; s.bytes += n.bytes; }
    }
    for (int k = 0; k < PK_COUNT; ++k)
        if (c.prof[k].ev.size() >= 8192) prof_drain(c, k);
    return SARAS_OK;
}

static const char *kProfNames[PK_COUNT] = {
    "mg_smooth_fp64", "mg_smooth_fp32", "mg_residual_fp64", "mg_residual_fp32", "mg_restrict_fp64", "mg_restrict_fp32",
    "mg_prolong_fp64", "mg_prolong_fp32", "refine_residual_fp64", "refine_update_fp64", "nse_rhs", "cn_jacobi",
    "projection", "divergence", "conv3d_fwd_tcgen05", "conv3d_bwd_tcgen05", "initial_guess"};

// ------------------------------------------------------------------ yaml
static std::string trim(const std::string &s) {
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}
static std::string unquote(const std::string &s) {
    std::string t = trim(s);
    if (t.size() >= 2 && ((t.front() == '"' && t.back() == '"') || (t.front() == '\'' && t.back() == '\''))) return t.substr(1, t.size() - 2);
    return t;
}

// Reads the flat two-level YAML of input/parameters.yaml: "Section": then
// indented "Key": value pairs, '#' comments and one folded block scalar.
static bool read_yaml(const char *path, std::map<std::string, std::string> &kv, std::string &err) {
    std::ifstream in(path);
    if (!in) { err = std::string("cannot open ") + path; return false; }
    std::string line, section;
    int blockIndent = -1;
    std::string blockKey;
    while (std::getline(in, line)) {
        std::string raw = line;
        size_t hash = std::string::npos;
        bool inq = false;
        for (size_t q = 0; q < raw.size(); ++q) {
            if (raw[q] == '"') inq = !inq;
            if (raw[q] == '#' && !inq) { hash = q; break; }
        }
        if (hash != std::string::npos) raw = raw.substr(0, hash);
        if (trim(raw).empty()) continue;
        int indent = 0;
        while (indent < (int)raw.size() && (raw[indent] == ' ' || raw[indent] == '\t')) ++indent;
        if (blockIndent >= 0) {
            if (indent > blockIndent) { kv[blockKey] += trim(raw) + "\n"; continue; }
            blockIndent = -1;
        }
        std::string t = trim(raw);
        size_t colon = std::string::npos;
        inq = false;
        for (size_t q = 0; q < t.size(); ++q) {
            if (t[q] == '"') inq = !inq;
            if (t[q] == ':' && !inq) { colon = q; break; }
        }
        if (colon == std::string::npos) { err = "malformed line: " + line; return false; }
        std::string key = unquote(t.substr(0, colon));
        std::string val = trim(t.substr(colon + 1));
        if (indent == 0) { section = key; continue; }
        std::string full = section + "/" + key;
        if (val == ">" || val == "|") { blockIndent = indent; blockKey = full; kv[full] = ""; continue; }
        kv[full] = unquote(val);
    }
    return true;
}

static bool to_int(const std::string &s, int &out) {
    char *e = nullptr;
    long v = std::strtol(s.c_str(), &e, 10);
    if (e == s.c_str() || *e != '\0') return false;
    out = (int)v;
    return true;
}
static bool to_double(const std::string &s, double &out) {
    char *e = nullptr;
    double v = std::strtod(s.c_str(), &e);
    if (e == s.c_str() || *e != '\0') return false;
    out = v;
    return true;
}
static bool to_bool(const std::string &s, int &out) {
    std::string t = s;
    std::transform(t.begin(), t.end(), t.begin(), ::tolower);
    if (t == "true" || t == "yes" || t == "on" || t == "1") { out = 1; return true; }
    if (t == "false" || t == "no" || t == "off" || t == "0") { out = 0; return true; }
    return false;
}

}  // namespace saras

using namespace saras;

extern "C" {

int saras_default_params(saras_params *p) {
    if (!p) return SARAS_BAD_ARG;
    std::memset(p, 0, sizeof(*p));
    p->probType = 2; p->icType = 1; p->rbcType = 1; p->forceType = 0;
    p->xPer = p->yPer = p->zPer = 1;
    p->Re = 1000.0; p->Ra = 1.0e4; p->Pr = 0.71; p->Ro = 12.0; p->Ta = 0.0;
    p->Lx = p->Ly = p->Lz = 1.0;
    p->nonHgBC = 0; p->patchRadius = 0.25;
    p->betaX = p->betaY = p->betaZ = 1.0;
    p->xInd = p->yInd = p->zInd = 5;
    p->nThreads = 1; p->npX = 1; p->npY = 1;
    p->dScheme = 1; p->iScheme = 1;
    p->cnTolerance = 1.0e-8;
    p->courantNumber = 0.1; p->tStp = 1.0e-3; p->tMax = 0.1;
    p->ioCnt = 1; p->solnFormat = 1; p->fwInt = 0.1; p->rsInt = 0.1; p->prInt = 0.1;
    p->vcDepth = 3; p->vcCount = 200; p->mgTolerance = 1.0e-8;
    p->gsSmooth = 0; p->preSmooth = 3; p->postSmooth = 3; p->resType = 1;
    p->mgMode = SARAS_MG_REFERENCE; p->mgTarget = 1.0e-8; p->mgMaxCycles = 200; p->mixedCycles = 1;
    p->guessMode = SARAS_GUESS_PREVIOUS; p->jacobiWeight = 1.0; p->seed = 42;
    return SARAS_OK;
}

static int fail(char *err, int errlen, const std::string &msg, int code) {
    if (err && errlen > 0) { std::strncpy(err, msg.c_str(), errlen - 1); err[errlen - 1] = 0; }
    set_error(msg);
    return code;
}

// parser::parseYAML (parser.cc:158-236) and parser::checkData (parser.cc:250-352).
int saras_parse_yaml(const char *path, saras_params *p, char *err, int errlen) {
    if (!path || !p) return fail(err, errlen, "null argument", SARAS_BAD_ARG);
    saras_default_params(p);
    std::map<std::string, std::string> kv;
    std::string e;
    if (!read_yaml(path, kv, e)) return fail(err, errlen, e, SARAS_BAD_CONFIG);
    struct IK { const char *k; int *v; };
    struct DK { const char *k; double *v; };
    struct BK { const char *k; int *v; };
    IK ints[] = {{"Program/Problem Type", &p->probType}, {"Program/Initial Condition", &p->icType}, {"Program/RBC Type", &p->rbcType},
                 {"Program/Force", &p->forceType}, {"Mesh/X Index", &p->xInd}, {"Mesh/Y Index", &p->yInd}, {"Mesh/Z Index", &p->zInd},
                 {"Parallel/Number of OMP threads", &p->nThreads}, {"Parallel/X Number of Procs", &p->npX},
                 {"Parallel/Y Number of Procs", &p->npY}, {"Solver/Differentiation Scheme", &p->dScheme},
                 {"Solver/Integration Scheme", &p->iScheme}, {"Solver/I/O Count", &p->ioCnt}, {"Solver/Solution Format", &p->solnFormat},
                 {"Multigrid/V-Cycle Depth", &p->vcDepth}, {"Multigrid/V-Cycle Count", &p->vcCount},
                 {"Multigrid/Smoothing Method", &p->gsSmooth}, {"Multigrid/Pre-Smoothing Count", &p->preSmooth},
                 {"Multigrid/Post-Smoothing Count", &p->postSmooth}, {"Multigrid/Residual Type", &p->resType},
                 {"GB300/Multigrid Mode", &p->mgMode}, {"GB300/Max V-Cycles", &p->mgMaxCycles},
                 {"GB300/Mixed Inner Cycles", &p->mixedCycles}, {"GB300/Guess Mode", &p->guessMode}, {"GB300/Seed", &p->seed},
                 {"GB300/Fast Kernels", &p->fastKernels}, {"GB300/Smoother", &p->smoother},
                 {"GB300/Coarse Smoothing Count", &p->coarseSmooth}, {"GB300/Coarse Cycles", &p->coarseCycles}};
    DK dbls[] = {{"Program/Reynolds Number", &p->Re}, {"Program/Rossby Number", &p->Ro}, {"Program/Rayleigh Number", &p->Ra},
                 {"Program/Prandtl Number", &p->Pr}, {"Program/Taylor Number", &p->Ta}, {"Program/X Length", &p->Lx},
                 {"Program/Y Length", &p->Ly}, {"Program/Z Length", &p->Lz}, {"Program/Plate Radius", &p->patchRadius},
                 {"Mesh/X Beta", &p->betaX}, {"Mesh/Y Beta", &p->betaY}, {"Mesh/Z Beta", &p->betaZ},
                 {"Solver/Solve Tolerance", &p->cnTolerance}, {"Solver/Courant Number", &p->courantNumber},
                 {"Solver/Time-Step", &p->tStp}, {"Solver/Final Time", &p->tMax}, {"Solver/Solution Write Interval", &p->fwInt},
                 {"Solver/Restart Write Interval", &p->rsInt}, {"Solver/Probe Time Interval", &p->prInt},
                 {"Multigrid/Solve Tolerance", &p->mgTolerance}, {"GB300/Residual Target", &p->mgTarget},
                 {"GB300/Jacobi Weight", &p->jacobiWeight}};
    BK bools[] = {{"Program/Heating Plate", &p->nonHgBC}, {"Solver/Restart Run", &p->restartFlag},
                  {"Solver/Use CFL Condition", &p->useCFL}, {"Solver/Record Probes", &p->readProbes},
                  {"Multigrid/Print Residual", &p->printResidual}, {"GB300/Test Poisson", &p->testPoisson}};
    const char *required[] = {"Program/Problem Type", "Program/Domain Type", "Mesh/Mesh Type", "Mesh/X Index", "Mesh/Y Index",
                              "Mesh/Z Index", "Solver/Time-Step", "Solver/Final Time", "Multigrid/V-Cycle Depth"};
    for (const char *r : required)
        if (!kv.count(r)) return fail(err, errlen, std::string("missing key ") + r, SARAS_BAD_CONFIG);
    for (auto &x : ints) if (kv.count(x.k) && !to_int(kv[x.k], *x.v)) return fail(err, errlen, std::string("bad integer for ") + x.k, SARAS_BAD_CONFIG);
    for (auto &x : dbls) if (kv.count(x.k) && !to_double(kv[x.k], *x.v)) return fail(err, errlen, std::string("bad number for ") + x.k, SARAS_BAD_CONFIG);
    for (auto &x : bools) if (kv.count(x.k) && !to_bool(kv[x.k], *x.v)) return fail(err, errlen, std::string("bad boolean for ") + x.k, SARAS_BAD_CONFIG);
    std::string domain = kv["Program/Domain Type"], mesh = kv["Mesh/Mesh Type"];
    // parser::checkData (parser.cc:250-352)
    // "Y Index" 0 selects the 2D (PLANAR) solver at run time (parser.cc:252-262)
    if (p->npX < 1) p->npX = 1;
    if (p->npY < 1) p->npY = 1;
    if (domain.size() != 3) return fail(err, errlen, "Domain type string is not correct", SARAS_BAD_CONFIG);
    if (mesh.size() != 3) return fail(err, errlen, "Mesh type string is not correct", SARAS_BAD_CONFIG);
    if (p->tStp > p->tMax) return fail(err, errlen, "Time step is larger than the maximum duration assigned for simulation", SARAS_BAD_CONFIG);
    if (p->resType > 2) return fail(err, errlen, "The specified value for printing error at end of V-Cycles is not defined", SARAS_BAD_CONFIG);
    // parser::setPeriodicity / setGrids (parser.cc:366-414)
    p->xPer = domain[0] != 'N'; p->yPer = domain[1] != 'N'; p->zPer = domain[2] != 'N';
    auto g = [](char ch) { return ch == 'S' ? 1 : ch == 'D' ? 2 : 0; };
    p->xGrid = g(mesh[0]); p->yGrid = g(mesh[1]); p->zGrid = g(mesh[2]);
    // One GPU runs the whole domain (np = 1 semantics); the decomposition check
    // uses the full grid.
    int coarsest = (int)std::pow(2, p->vcDepth + 1);
    if ((int)std::pow(2, p->xInd) < coarsest || (p->yInd != 0 && (int)std::pow(2, p->yInd) < coarsest) || (int)std::pow(2, p->zInd) < coarsest)
        return fail(err, errlen, "The grid size is too coarse to reach the V-Cycle depth specified", SARAS_BAD_CONFIG);
    return SARAS_OK;
}

static int validate(const saras_params *p, std::string &why) {
    const bool planar = p->yInd == 0;   // the 2D solver
    if (p->xInd < 2 || (p->yInd < 2 && !planar) || p->zInd < 2 || p->xInd > 11 || p->yInd > 11 || p->zInd > 11) { why = "grid index out of range (2..11; Y Index 0 for 2D)"; return SARAS_BAD_CONFIG; }
    if (p->vcDepth < 1) { why = "V-Cycle Depth must be >= 1"; return SARAS_BAD_CONFIG; }
    int coarsest = (int)std::pow(2, p->vcDepth + 1);
    if ((1 << p->xInd) < coarsest || (!planar && (1 << p->yInd) < coarsest) || (1 << p->zInd) < coarsest) { why = "grid too coarse for the V-Cycle depth"; return SARAS_BAD_CONFIG; }
    // 2D runs the drop-in form (the GB300 extensions are 3D)
    if (planar && (p->mgMode != SARAS_MG_REFERENCE || p->fastKernels != 0 || p->guessMode != SARAS_GUESS_PREVIOUS || p->testPoisson)) {
        why = "the 2D solver (Y Index 0) runs in the drop-in mode only: Multigrid Mode 0, Fast Kernels 0, Guess Mode 0, no Test Poisson";
        return SARAS_BAD_CONFIG;
    }
    if (p->xGrid < 0 || p->xGrid > 2 || p->yGrid < 0 || p->yGrid > 2 || p->zGrid < 0 || p->zGrid > 2) { why = "bad grid type"; return SARAS_BAD_CONFIG; }
    // Mesh Type 'D' (double-sided tangent-hyperbolic stretching, grid.cc:442-519)
    // runs in the drop-in mode: the reference's multigrid and FP64 kernels read
    // the metric arrays at every point; the GB300 extensions assume uniform
    // metrics.  ('S', single-sided, builds a uniform grid in the reference,
    // grid.cc:117-131, and does here.)
    const bool stretched = p->xGrid == 2 || (p->yGrid == 2 && !planar) || p->zGrid == 2;
    if (stretched && (p->mgMode != SARAS_MG_REFERENCE || p->fastKernels != 0 || p->guessMode != SARAS_GUESS_PREVIOUS || p->testPoisson)) {
        why = "stretched meshes (Mesh Type 'D') run in the drop-in mode only: Multigrid Mode 0, Fast Kernels 0, Guess Mode 0, no Test Poisson";
        return SARAS_BAD_CONFIG;
    }
    if ((p->xGrid == 2 && !(p->betaX > 0)) || (p->yGrid == 2 && !(p->betaY > 0)) || (p->zGrid == 2 && !(p->betaZ > 0))) {
        why = "the Beta of a stretched axis must be positive";
        return SARAS_BAD_CONFIG;
    }
    if (p->dScheme != 1) { why = "Undefined finite differencing scheme"; return SARAS_BAD_CONFIG; }
    if (p->gsSmooth < 0 || p->gsSmooth > 1) { why = "Smoothing Method must be 0 (Jacobi) or 1 (Gauss-Seidel)"; return SARAS_BAD_CONFIG; }
    if (p->nonHgBC) { why = "heating-plate boundary condition is not supported"; return SARAS_BAD_CONFIG; }
    if (p->probType >= 5 && (p->rbcType < 1 || p->rbcType > 4)) { why = "undefined RBC Type"; return SARAS_BAD_CONFIG; }
    if (p->tStp <= 0 || p->Re <= 0 || p->Lx <= 0 || p->Ly <= 0 || p->Lz <= 0) { why = "non-positive time step, Re or length"; return SARAS_BAD_CONFIG; }
    if (p->mgMode < 0 || p->mgMode > 2) { why = "bad multigrid mode"; return SARAS_BAD_CONFIG; }
    if (p->guessMode < SARAS_GUESS_PREVIOUS || p->guessMode > SARAS_GUESS_NETWORK) { why = "bad guess mode"; return SARAS_BAD_CONFIG; }
    if (p->fastKernels < 0 || p->fastKernels > 2) { why = "Fast Kernels must be 0, 1 or 2"; return SARAS_BAD_CONFIG; }
    if (p->smoother < 0 || p->smoother > 1) { why = "Smoother must be 0 (Jacobi) or 1 (Chebyshev)"; return SARAS_BAD_CONFIG; }
    if (p->smoother == 1 && (p->preSmooth > 16 || p->postSmooth > 16 || p->coarseSmooth > 16)) {
        why = "Chebyshev smoothing takes at most 16 sweeps a phase";
        return SARAS_BAD_CONFIG;
    }
    if (p->coarseSmooth < 0) { why = "negative Coarse Smoothing Count"; return SARAS_BAD_CONFIG; }
    // Target-mode cycles on a periodic axis need three sweeps a level at least:
    // V(1,1) cycles (weight 6/7, either smoother) stalled near 1e-5 of max|b|
    // on the 65^3 Taylor-Green vortex and then diverged; V(2,1), V(1,2) and
    // V(2,2) converged.
    if (p->mgMode != SARAS_MG_REFERENCE && (p->xPer || p->yPer || p->zPer) &&
        (p->preSmooth + p->postSmooth < 3 || (p->coarseSmooth > 0 && 2 * p->coarseSmooth < 3))) {
        why = "target multigrid modes on periodic axes need at least 3 smoothing sweeps a level (pre + post, or 2 x Coarse Smoothing Count)";
        return SARAS_BAD_CONFIG;
    }
    if (p->coarseCycles < 0 || p->coarseCycles > 4) { why = "Coarse Cycles must be 0 to 4"; return SARAS_BAD_CONFIG; }
    if (p->resType < 0 || p->resType > 2) { why = "bad residual type"; return SARAS_BAD_CONFIG; }
    return SARAS_OK;
}

int saras_create(const saras_params *p, saras_ctx **out) {
    if (!p || !out) return SARAS_BAD_ARG;
    *out = nullptr;
    std::string why;
    int s = validate(p, why);
    if (s) { set_error(why); return s; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device is visible; the GB300 solver has no CPU fallback");
        return SARAS_NO_DEVICE;
    }
    saras_ctx *h = new saras_ctx();
    Ctx &c = h->c;
    c.p = *p;
    cudaGetDevice(&c.dev);
    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        delete h;
        return SARAS_CUDA_ERROR;
    }
    c.guessMode = p->guessMode;
    s = fields_setup(c);
    if (!s) s = mg_setup(c);
    if (!s) {
        if (cudaStreamSynchronize(c.stream) != cudaSuccess) { set_error("setup failed"); s = SARAS_CUDA_ERROR; }
    }
    if (s) {
        if (c.err.empty()) c.err = g_err;
        set_error(c.err);
        saras_destroy(h);
        return s;
    }
    *out = h;
    return SARAS_OK;
}

int saras_destroy(saras_ctx *h) {
    if (!h) return SARAS_OK;
    Ctx &c = h->c;
    if (c.stream) cudaStreamSynchronize(c.stream);
    unet_free(c);
    mg_free(c);
    for (int f = 0; f < SARAS_NUM_FIELDS; ++f) cudaFree(c.f[f]);
    for (int q = 0; q < 4; ++q) cudaFree(c.scratch[q]);
    cudaFree(c.red); cudaFree(c.dscal); cudaFree(c.dflag); cudaFree(c.dmet);
    if (c.hscal) cudaFreeHost(c.hscal);
    for (int q = 0; q < 3; ++q) cudaFree(c.pHist[q]);
    cudaFree(c.cnp);
    cudaFree(c.probeBuf);
    for (int k = 0; k < PK_COUNT; ++k) for (cudaEvent_t e : c.prof[k].ev) cudaEventDestroy(e);
    for (cudaEvent_t e : c.evPool) cudaEventDestroy(e);
    for (int k = 0; k < 16; ++k) if (c.userEv[k]) cudaEventDestroy(c.userEv[k]);
    for (int q = 0; q < SARAS_NUM_FIELDS; ++q) if (c.copyStream[q]) cudaStreamDestroy(c.copyStream[q]);
    for (int q = 0; q <= SARAS_NUM_FIELDS; ++q) if (c.copyEvent[q]) cudaEventDestroy(c.copyEvent[q]);
    if (c.stream) cudaStreamDestroy(c.stream);
    delete h;
    return SARAS_OK;
}

const char *saras_last_error(const saras_ctx *h) {
    if (h && !h->c.err.empty()) return h->c.err.c_str();
    return g_err.c_str();
}

static long field_count(const Ctx &c, int f) {
    const FieldInfo &i = c.info[f];
    return (long)(i.n[0] + 2) * (i.n[1] + 2) * (i.n[2] + 2);
}

int saras_field_dims(const saras_ctx *h, int field, int dims[3]) {
    if (!h || !dims || field < 0 || field >= SARAS_NUM_FIELDS) return SARAS_BAD_ARG;
    for (int d = 0; d < 3; ++d) dims[d] = h->c.info[field].n[d] + 2;
    return SARAS_OK;
}

int saras_grid_coords(const saras_ctx *h, int axis, int staggered, double *out, int capacity, int *count) {
    if (!h || axis < 0 || axis > 2 || !count) return SARAS_BAD_ARG;
    const std::vector<double> &x = h->c.hcoord[axis][staggered ? 1 : 0];
    *count = (int)x.size();
    if (!out) return SARAS_OK;
    if (capacity < (int)x.size()) return SARAS_BAD_ARG;
    std::memcpy(out, x.data(), sizeof(double) * x.size());
    return SARAS_OK;
}

int saras_upload(saras_ctx *h, int field, const double *host) {
    if (!h || !host || field < 0 || field >= SARAS_NUM_FIELDS) return SARAS_BAD_ARG;
    Ctx &c = h->c;
    SARAS_CUDA_TRY(cudaMemcpyAsync(c.f[field], host, sizeof(double) * field_count(c, field), cudaMemcpyHostToDevice, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return SARAS_OK;
}

int saras_download(saras_ctx *h, int field, double *host) {
    if (!h || !host || field < 0 || field >= SARAS_NUM_FIELDS) return SARAS_BAD_ARG;
    Ctx &c = h->c;
    SARAS_CUDA_TRY(cudaMemcpyAsync(host, c.f[field], sizeof(double) * field_count(c, field), cudaMemcpyDeviceToHost, c.stream));
    SARAS_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return SARAS_OK;
}

// Field copies on one stream each: every copy stream waits for the context
// stream's work so far, and (upload) the context stream waits for every copy.
// A field may appear once per call (two concurrent copies into one device
// buffer would race).  If issuing fails part way, the copies already issued
// are waited for before returning, so no copy still reads or writes the
// caller's host buffers when the error comes back.
static int copy_fields(Ctx &c, int n, const int *fields, const void *const *hosts, bool up) {
    if (n < 0 || n > SARAS_NUM_FIELDS || (n > 0 && (!fields || !hosts))) return SARAS_BAD_ARG;
    bool seen[SARAS_NUM_FIELDS] = {};
    for (int q = 0; q < n; ++q) {
        if (fields[q] < 0 || fields[q] >= SARAS_NUM_FIELDS || !hosts[q]) return SARAS_BAD_ARG;
        if (seen[fields[q]]) { c.err = "a field appears twice in one copy call"; set_error(c.err); return SARAS_BAD_ARG; }
        seen[fields[q]] = true;
    }
    for (int q = 0; q <= n; ++q)
        if (!c.copyEvent[q]) SARAS_CUDA_TRY(cudaEventCreateWithFlags(&c.copyEvent[q], cudaEventDisableTiming));
    for (int q = 0; q < n; ++q)
        if (!c.copyStream[q]) SARAS_CUDA_TRY(cudaStreamCreateWithFlags(&c.copyStream[q], cudaStreamNonBlocking));
    SARAS_CUDA_TRY(cudaEventRecord(c.copyEvent[n], c.stream));
    int issued = 0;
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < n && e == cudaSuccess; ++q) {
        cudaStream_t st = c.copyStream[q];
        size_t bytes = sizeof(double) * field_count(c, fields[q]);
        e = cudaStreamWaitEvent(st, c.copyEvent[n], 0);
        if (e == cudaSuccess) {
            issued = q + 1;
            e = up ? cudaMemcpyAsync(c.f[fields[q]], hosts[q], bytes, cudaMemcpyHostToDevice, st)
                   : cudaMemcpyAsync(const_cast<void *>(hosts[q]), c.f[fields[q]], bytes, cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess) e = cudaEventRecord(c.copyEvent[q], st);
    }
    if (e != cudaSuccess) {
        for (int q = 0; q < issued; ++q) cudaStreamSynchronize(c.copyStream[q]);
        set_error(std::string("field copy: ") + cudaGetErrorString(e));
        return SARAS_CUDA_ERROR;
    }
    for (int q = 0; q < n; ++q) {
        SARAS_CUDA_TRY(cudaStreamWaitEvent(c.stream, c.copyEvent[q], 0));
        SARAS_CUDA_TRY(cudaEventSynchronize(c.copyEvent[q]));
    }
    return SARAS_OK;
}

int saras_upload_fields(saras_ctx *h, int n, const int *fields, const double *const *hosts) {
    if (!h) return SARAS_BAD_ARG;
    return copy_fields(h->c, n, fields, reinterpret_cast<const void *const *>(hosts), true);
}

int saras_download_fields(saras_ctx *h, int n, const int *fields, double *const *hosts) {
    if (!h) return SARAS_BAD_ARG;
    return copy_fields(h->c, n, fields, reinterpret_cast<const void *const *>(hosts), false);
}

int saras_synchronize(saras_ctx *h) {
    if (!h) return SARAS_BAD_ARG;
    SARAS_CUDA_TRY(cudaStreamSynchronize(h->c.stream));
    return SARAS_OK;
}

long long saras_launch_count(const saras_ctx *h) { return h ? h->c.launches : 0; }
int saras_plane_tma_active(const saras_ctx *h) { return h && h->c.planeOk ? 1 : 0; }

#define CTX_OR_FAIL(h) do { if (!h) return SARAS_BAD_ARG; } while (0)

int saras_apply_bc(saras_ctx *h, int field) { CTX_OR_FAIL(h); return apply_bc(h->c, field); }
int saras_sync_field(saras_ctx *h, int field) { CTX_OR_FAIL(h); return sync_field(h->c, field); }
int saras_vfield_compute_diff(saras_ctx *h) { CTX_OR_FAIL(h); return vfield_compute_diff(h->c); }
int saras_vfield_compute_nlin(saras_ctx *h) { CTX_OR_FAIL(h); return vfield_compute_nlin(h->c); }
int saras_sfield_gradient(saras_ctx *h, int sf) { CTX_OR_FAIL(h); return sfield_gradient(h->c, sf); }
int saras_vfield_divergence(saras_ctx *h) { CTX_OR_FAIL(h); return vfield_divergence(h->c, nullptr, false); }
int saras_tfield_compute_diff(saras_ctx *h) { CTX_OR_FAIL(h); return tfield_compute_diff(h->c); }
int saras_tfield_compute_nlin(saras_ctx *h) { CTX_OR_FAIL(h); return tfield_compute_nlin(h->c); }
int saras_axpby(saras_ctx *h, int dst, double a, int src, double b) { CTX_OR_FAIL(h); return axpby(h->c, dst, a, src, b); }

int saras_cn_solve(saras_ctx *h, int component, int *iters, double *max_error) {
    CTX_OR_FAIL(h);
    for (int &q : h->c.n0Fresh) q = 0;   // nseRHS may have been set by the caller
    return cn_solve(h->c, component, iters, max_error);
}

int saras_mg_solve(saras_ctx *h, int *vcycles, double *residual) {
    CTX_OR_FAIL(h);
    return mg_solve(h->c, vcycles, residual, nullptr);
}

int saras_mg_set_mode(saras_ctx *h, int mode, double target, int max_cycles) {
    CTX_OR_FAIL(h);
    if (mode < 0 || mode > 2 || !(target > 0) || max_cycles < 1) return SARAS_BAD_ARG;
    if (h->c.stretched && mode != SARAS_MG_REFERENCE) { set_error("stretched meshes run the reference multigrid only"); return SARAS_BAD_CONFIG; }
    h->c.mgMode = mode; h->c.mgTarget = target; h->c.mgMaxCycles = max_cycles;
    h->c.p.mgMode = mode; h->c.p.mgTarget = target; h->c.p.mgMaxCycles = max_cycles;
    return SARAS_OK;
}

int saras_time_advance(saras_ctx *h, saras_step_stats *stats) {
    CTX_OR_FAIL(h);
    return time_advance(h->c, stats);
}

// parser::parseProbes / testProbes (parser.cc:424-575): each "[x, y, z]" set
// of the "Probes" value gives one index list per axis, an integer or a range
// "start:end:count" expanded to start + round(i (end - start) / (count - 1));
// the probes are the sets' Cartesian products (x outermost), in set order.
// Every index must lie in 0 .. 2^index + 1 of its axis.
static bool expand_probes(const std::string &spec, const int ind[3], std::vector<int> &out, std::string &err) {
    size_t pos = 0;
    while (true) {
        size_t lb = spec.find('[', pos);
        if (lb == std::string::npos) break;
        size_t rb = spec.find(']', lb);
        if (rb == std::string::npos) { err = "unbalanced [ in Probes"; return false; }
        const std::string set = spec.substr(lb + 1, rb - lb - 1);
        pos = rb + 1;
        std::vector<std::vector<int>> lists;
        std::stringstream ss(set);
        std::string item;
        while (std::getline(ss, item, ',')) {
            item = trim(item);
            std::vector<int> v;
            if (item.find(':') == std::string::npos) {
                int x;
                if (!to_int(item, x)) { err = "bad probe index '" + item + "'"; return false; }
                v.push_back(x);
            } else {
                int a, b, n;
                std::string t = item;
                size_t c1 = t.find(':'), c2 = t.find(':', c1 + 1);
                if (c2 == std::string::npos || !to_int(trim(t.substr(0, c1)), a) || !to_int(trim(t.substr(c1 + 1, c2 - c1 - 1)), b) ||
                    !to_int(trim(t.substr(c2 + 1)), n) || a < 0 || b < 0 || n < 0) {
                    err = "bad probe range '" + item + "'";
                    return false;
                }
                if (a == b || n == 1) v.push_back(a);
                else
                    for (int i = 0; i < n; ++i) {
                        double inc = ((double)b - (double)a) / ((double)n - 1.0);
                        v.push_back(a + (int)std::round((double)i * inc));
                    }
            }
            lists.push_back(v);
        }
        if (lists.size() != 3) {
            err = "Number of indices for the probe(s) [" + set + "] does not match dimensionality of problem";
            return false;
        }
        for (int x : lists[0])
            for (int y : lists[1])
                for (int z : lists[2]) { out.push_back(x); out.push_back(y); out.push_back(z); }
    }
    const char *axis = "XYZ";
    for (size_t q = 0; q < out.size(); ++q) {
        int d = (int)(q % 3), lim = (1 << ind[d]) + 1;
        if (out[q] < 0 || out[q] > lim) {
            err = std::string("The ") + axis[d] + " index of a probe lies outside the bounds of the domain";
            return false;
        }
    }
    return true;
}

int saras_parse_probes(const char *path, int *ijk, int capacity, int *count, char *err, int errlen) {
    if (!path || !count || capacity < 0 || (capacity > 0 && !ijk)) return SARAS_BAD_ARG;
    saras_params p;
    int s = saras_parse_yaml(path, &p, err, errlen);
    if (s) return s;
    std::map<std::string, std::string> kv;
    std::string e;
    if (!read_yaml(path, kv, e)) return fail(err, errlen, e, SARAS_BAD_CONFIG);
    std::vector<int> out;
    const int ind[3] = {p.xInd, p.yInd, p.zInd};
    if (kv.count("Solver/Probes") && !expand_probes(kv["Solver/Probes"], ind, out, e)) return fail(err, errlen, e, SARAS_BAD_CONFIG);
    *count = (int)(out.size() / 3);
    for (int q = 0; q < std::min(*count, capacity); ++q)
        for (int d = 0; d < 3; ++d) ijk[3 * q + d] = out[3 * q + d];
    return SARAS_OK;
}

// Restart files (writer::writeRestart, writer.cc:455-540, written every
// "Restart Write Interval", hydro_d3.cc:229-231; reader::readData,
// reader.cc:213-296): "Time" and the cores of Vx, Vy, Vz, P (and T with the
// scalar solver) with the reference restart file's dataset names and core
// shapes, in a raw little-endian container (no HDF5 library is linked):
//   "SARASRST", int32 version 1, int32 field count n, float64 time,
//   n x {char name[16] (NUL-padded), int32 core points along x, y, z},
//   then the n cores as float64 in C order (z fastest), in header order.
static const char kRestartMagic[8] = {'S', 'A', 'R', 'A', 'S', 'R', 'S', 'T'};

static std::vector<int> restart_fields(const Ctx &c) {
    std::vector<int> f = {SARAS_FIELD_VX, SARAS_FIELD_VY, SARAS_FIELD_VZ, SARAS_FIELD_P};
    if (c.scalar) f.push_back(SARAS_FIELD_T);
    return f;
}
static const char *restart_name(int f) {
    switch (f) {
        case SARAS_FIELD_VX: return "Vx";
        case SARAS_FIELD_VY: return "Vy";
        case SARAS_FIELD_VZ: return "Vz";
        case SARAS_FIELD_P: return "P";
        default: return "T";
    }
}

int saras_write_restart(saras_ctx *h, const char *path, double time) {
    if (!h || !path) return SARAS_BAD_ARG;
    Ctx &c = h->c;
    const std::vector<int> fields = restart_fields(c);
    FILE *fp = std::fopen(path, "wb");
    if (!fp) { c.err = std::string("cannot create ") + path; return SARAS_BAD_ARG; }
    int32_t hdr[2] = {1, (int32_t)fields.size()};
    bool ok = std::fwrite(kRestartMagic, 1, 8, fp) == 8 && std::fwrite(hdr, sizeof(int32_t), 2, fp) == 2 &&
              std::fwrite(&time, sizeof(double), 1, fp) == 1;
    for (int f : fields) {
        char name[16] = {0};
        std::strncpy(name, restart_name(f), 15);
        int32_t dims[3] = {c.info[f].n[0], c.info[f].n[1], c.info[f].n[2]};
        ok = ok && std::fwrite(name, 1, 16, fp) == 16 && std::fwrite(dims, sizeof(int32_t), 3, fp) == 3;
    }
    std::vector<double> pad, core;
    for (int f : fields) {
        if (!ok) break;
        const int n0 = c.info[f].n[0], n1 = c.info[f].n[1], n2 = c.info[f].n[2];
        pad.resize(field_count(c, f));
        int s = saras_download(h, f, pad.data());
        if (s) { std::fclose(fp); return s; }
        core.resize((size_t)n0 * n1 * n2);
        for (int i = 0; i < n0; ++i)
            for (int j = 0; j < n1; ++j)
                std::memcpy(&core[((size_t)i * n1 + j) * n2], &pad[((size_t)(i + 1) * (n1 + 2) + (j + 1)) * (n2 + 2) + 1],
                            sizeof(double) * n2);
        ok = std::fwrite(core.data(), sizeof(double), core.size(), fp) == core.size();
    }
    if (std::fclose(fp) != 0) ok = false;
    if (!ok) { c.err = std::string("writing ") + path + " failed"; return SARAS_BAD_ARG; }
    return SARAS_OK;
}

int saras_read_restart(saras_ctx *h, const char *path, double *time) {
    if (!h || !path) return SARAS_BAD_ARG;
    Ctx &c = h->c;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) { c.err = std::string("Restart flag is true, but could not open restart file ") + path; return SARAS_BAD_CONFIG; }
    char magic[8];
    int32_t hdr[2];
    double t = 0.0;
    bool ok = std::fread(magic, 1, 8, fp) == 8 && std::memcmp(magic, kRestartMagic, 8) == 0 && std::fread(hdr, sizeof(int32_t), 2, fp) == 2 &&
              hdr[0] == 1 && hdr[1] > 0 && hdr[1] <= SARAS_NUM_FIELDS && std::fread(&t, sizeof(double), 1, fp) == 1;
    std::vector<std::string> names;
    std::vector<std::array<int32_t, 3>> dims;
    for (int q = 0; ok && q < hdr[1]; ++q) {
        char name[17] = {0};
        std::array<int32_t, 3> d;
        ok = std::fread(name, 1, 16, fp) == 16 && std::fread(d.data(), sizeof(int32_t), 3, fp) == 3 && d[0] > 0 && d[1] > 0 && d[2] > 0;
        names.push_back(name);
        dims.push_back(d);
    }
    if (!ok) { std::fclose(fp); c.err = std::string(path) + " is not a restart file of this format"; return SARAS_BAD_CONFIG; }
    const long dataStart = std::ftell(fp);
    // reader::restartCheck (reader.cc:338-399): every field present with the context's core shape
    std::vector<double> pad;
    for (int f : restart_fields(c)) {
        long off = dataStart;
        int q = 0;
        for (; q < (int)names.size() && names[q] != restart_name(f); ++q) off += (long)sizeof(double) * dims[q][0] * dims[q][1] * dims[q][2];
        const int n0 = c.info[f].n[0], n1 = c.info[f].n[1], n2 = c.info[f].n[2];
        if (q == (int)names.size() || dims[q][0] != n0 || dims[q][1] != n1 || dims[q][2] != n2) {
            std::fclose(fp);
            c.err = std::string("restart file does not match the grid: field ") + restart_name(f);
            return SARAS_BAD_CONFIG;
        }
        pad.assign(field_count(c, f), 0.0);
        if (std::fseek(fp, off, SEEK_SET) != 0) ok = false;
        for (int i = 0; ok && i < n0; ++i)
            for (int j = 0; ok && j < n1; ++j)
                ok = std::fread(&pad[((size_t)(i + 1) * (n1 + 2) + (j + 1)) * (n2 + 2) + 1], sizeof(double), n2, fp) == (size_t)n2;
        if (!ok) { std::fclose(fp); c.err = std::string("reading ") + path + " failed"; return SARAS_BAD_CONFIG; }
        int s = saras_upload(h, f, pad.data());
        if (s) { std::fclose(fp); return s; }
    }
    std::fclose(fp);
    if (time) *time = t;
    return SARAS_OK;
}

int saras_unet_shape(saras_ctx *h, long long *nparam, int dims[3]) {
    CTX_OR_FAIL(h);
    return unet_shape(h->c, nparam, dims);
}

int saras_unet_grad_check(saras_ctx *h, const float *feat, const float *target, const float *params, float *out, double *loss,
                          float *grad) {
    CTX_OR_FAIL(h);
    if (!feat || !target) return SARAS_BAD_ARG;
    return unet_grad_check(h->c, feat, target, params, out, loss, grad);
}

int saras_compute_tstp(saras_ctx *h, double *dt) {
    CTX_OR_FAIL(h);
    if (!dt) return SARAS_BAD_ARG;
    return compute_tstp(h->c, dt);
}

int saras_set_dt(saras_ctx *h, double dt) {
    CTX_OR_FAIL(h);
    if (!(dt > 0.0) || !std::isfinite(dt)) return SARAS_BAD_ARG;
    h->c.dt = dt;
    return SARAS_OK;
}

int saras_probe(saras_ctx *h, int n, const int *ijk, int nfields, const int *fields, double *out) {
    CTX_OR_FAIL(h);
    return probe(h->c, n, ijk, nfields, fields, out);
}

int saras_diagnostics(saras_ctx *h, double *energy, double *max_div, double *nusselt) {
    CTX_OR_FAIL(h);
    return diagnostics(h->c, energy, max_div, nusselt);
}

int saras_mg_test_prolong(saras_ctx *h, double *err) { CTX_OR_FAIL(h); if (!err) return SARAS_BAD_ARG; return mg_test_prolong(h->c, err); }
int saras_mg_test_transfer(saras_ctx *h, double *err) { CTX_OR_FAIL(h); if (!err) return SARAS_BAD_ARG; return mg_test_transfer(h->c, err); }
int saras_mg_test_periodic(saras_ctx *h, double *err) { CTX_OR_FAIL(h); if (!err) return SARAS_BAD_ARG; return mg_test_periodic(h->c, err); }
int saras_hydro_test_periodic(saras_ctx *h, double *err) { CTX_OR_FAIL(h); if (!err) return SARAS_BAD_ARG; return hydro_test_periodic(h->c, err); }

int saras_mg_level_dims(const saras_ctx *h, int level, int dims[3]) {
    if (!h || !dims || level < 0 || level > h->c.depth) return SARAS_BAD_ARG;
    for (int d = 0; d < 3; ++d) dims[d] = h->c.lv[level].n[d] + 3;
    return SARAS_OK;
}
int saras_mg_set_level(saras_ctx *h, int level, int which, const double *host) { CTX_OR_FAIL(h); if (!host) return SARAS_BAD_ARG; return mg_set_level(h->c, level, which, host); }
int saras_mg_get_level(saras_ctx *h, int level, int which, double *host) { CTX_OR_FAIL(h); if (!host) return SARAS_BAD_ARG; return mg_get_level(h->c, level, which, host); }
int saras_mg_smooth(saras_ctx *h, int level, int count) { CTX_OR_FAIL(h); return mg_smooth_level(h->c, level, count); }
int saras_mg_restrict(saras_ctx *h, int level) { CTX_OR_FAIL(h); return mg_restrict_level(h->c, level); }
int saras_mg_prolong_add(saras_ctx *h, int level) { CTX_OR_FAIL(h); return mg_prolong_level(h->c, level); }
int saras_mg_compute_error(saras_ctx *h, int norm, double *err) {
    CTX_OR_FAIL(h);
    if (!err || norm < 1 || norm > 2) return SARAS_BAD_ARG;
    return mg_compute_error(h->c, norm, err);
}

int saras_unet_collect(saras_ctx *h) { CTX_OR_FAIL(h); return unet_collect(h->c); }
int saras_unet_train(saras_ctx *h, int iters, double lr, double *loss) { CTX_OR_FAIL(h); return unet_train(h->c, iters, lr, loss); }
int saras_unet_infer(saras_ctx *h, int field_out) {
    CTX_OR_FAIL(h);
    if (field_out != SARAS_FIELD_PP) return SARAS_BAD_ARG;
    return unet_infer(h->c, h->c.f[SARAS_FIELD_PP]);
}
int saras_set_guess_mode(saras_ctx *h, int mode) {
    CTX_OR_FAIL(h);
    if (mode < SARAS_GUESS_PREVIOUS || mode > SARAS_GUESS_NETWORK) return SARAS_BAD_ARG;
    if (h->c.stretched && mode != SARAS_GUESS_PREVIOUS) { set_error("stretched meshes take the previous pressure as the guess"); return SARAS_BAD_CONFIG; }
    h->c.guessMode = mode;
    return SARAS_OK;
}

int saras_profile_enable(saras_ctx *h, int kernel_id, int enable) {
    if (!h || kernel_id < 0 || kernel_id >= PK_COUNT) return SARAS_BAD_ARG;
    ProfSlot &s = h->c.prof[kernel_id];
    prof_drain(h->c, kernel_id);
    if (enable) { s.launches = 0; s.bytes = 0; s.ms = 0; }
    s.enabled = enable != 0;
    while (enable && h->c.evPool.size() < 1024) {   // events for a few hundred timed launches up front
        cudaEvent_t e = nullptr;
        SARAS_CUDA_TRY(cudaEventCreate(&e));
        h->c.evPool.push_back(e);
    }
    return SARAS_OK;
}

int saras_profile_read(saras_ctx *h, int kernel_id, long long *launches, double *total_ms, double *bytes) {
    if (!h || kernel_id < 0 || kernel_id >= PK_COUNT) return SARAS_BAD_ARG;
    SARAS_CUDA_TRY(cudaStreamSynchronize(h->c.stream));
    prof_drain(h->c, kernel_id);
    const ProfSlot &s = h->c.prof[kernel_id];
    if (launches) *launches = s.launches;
    if (total_ms) *total_ms = s.ms;
    if (bytes) *bytes = s.bytes;
    return SARAS_OK;
}

int saras_profile_sample(saras_ctx *h, int every) {
    if (!h || every < 1) return SARAS_BAD_ARG;
    h->c.profEvery = every;
    h->c.profReplays = 0;
    return SARAS_OK;
}

const char *saras_profile_name(int kernel_id) {
    if (kernel_id < 0 || kernel_id >= PK_COUNT) return "";
    return kProfNames[kernel_id];
}

int saras_profile_count(void) { return PK_COUNT; }

int saras_event_record(saras_ctx *h, int slot) {
    if (!h || slot < 0 || slot >= 16) return SARAS_BAD_ARG;
    Ctx &c = h->c;
    if (!c.userEv[slot]) SARAS_CUDA_TRY(cudaEventCreate(&c.userEv[slot]));
    SARAS_CUDA_TRY(cudaEventRecord(c.userEv[slot], c.stream));
    return SARAS_OK;
}

int saras_event_elapsed(saras_ctx *h, int a, int b, double *ms) {
    if (!h || !ms || a < 0 || a >= 16 || b < 0 || b >= 16) return SARAS_BAD_ARG;
    Ctx &c = h->c;
    if (!c.userEv[a] || !c.userEv[b]) return SARAS_BAD_ARG;
    SARAS_CUDA_TRY(cudaEventSynchronize(c.userEv[b]));
    float f = 0;
    SARAS_CUDA_TRY(cudaEventElapsedTime(&f, c.userEv[a], c.userEv[b]));
    *ms = f;
    return SARAS_OK;
}

}  // extern "C"
