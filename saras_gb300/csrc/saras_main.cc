// saras_main.cc -- the SARAS executable on the GB300 library: the program of
// src/solvers/main.cc:49-157 with the solver's constructor and time loop
// (hydro_d3.cc:63-251, scalar_d3.cc:62-240) written over the C ABI of
// include/saras_gb300.h.  Host C++ only; every computation runs in the library.
//
//   saras_gb300_run [parameters.yaml] [output directory]
//
// Defaults: input/parameters.yaml and output/.  Writes TimeSeries.dat
// (tseries.cc:62-178, 195-246), ProbesData.dat when "Record Probes" is true
// (probes.cc:61-166) and restartFile.saras every "Restart Write Interval"
// (the datasets of writer::writeRestart, writer.cc:455-540, in the raw
// container of saras_write_restart); a "Restart Run" reads that file.  Solution
// files are not written.  Errors print the reference's message and exit 0, as
// the reference does.
#include <sys/stat.h>
#include <sys/time.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "saras_gb300.h"

namespace {

[[noreturn]] void abort_run(const std::string &msg) {
    std::cout << std::endl << msg << std::endl << std::endl;
    std::exit(0);
}

void check(int status, const saras_ctx *ctx, const char *what) {
    if (status == SARAS_OK) return;
    if (status == SARAS_NOT_CONVERGED) abort_run("ERROR: Jacobi iterations for solution of Vx not converging. Aborting");
    if (status == SARAS_DIVERGENCE_LIMIT) abort_run("ERROR: Divergence exceeds permissible limits. ABORTING");
    abort_run(std::string("ERROR: ") + what + ": " + saras_last_error(ctx));
}

struct Field {
    int dims[3];
    std::vector<double> v;
    double &at(int i, int j, int k) { return v[((size_t)(i + 1) * dims[1] + (j + 1)) * dims[2] + (k + 1)]; }
};

Field host_field(saras_ctx *ctx, int f) {
    Field h;
    check(saras_field_dims(ctx, f, h.dims), ctx, "field dimensions");
    h.v.assign((size_t)h.dims[0] * h.dims[1] * h.dims[2], 0.0);
    return h;
}

// taylorGreen::initializeField (taylorGreen.cc:54-100) over the padded arrays,
// with the library's coordinates (grid.cc:370-403 uniform, 442-519 stretched).
std::vector<double> coords(saras_ctx *ctx, int axis, int staggered) {
    int n = 0;
    check(saras_grid_coords(ctx, axis, staggered, nullptr, 0, &n), ctx, "grid coordinates");
    std::vector<double> x((size_t)n);
    check(saras_grid_coords(ctx, axis, staggered, x.data(), n, &n), ctx, "grid coordinates");
    return x;
}

void taylor_green(saras_ctx *ctx, const saras_params &p) {
    const double L[3] = {p.Lx, p.Ly, p.Lz};
    std::vector<double> xs = coords(ctx, 0, 1), xc = coords(ctx, 0, 0), ys = coords(ctx, 1, 1), yc = coords(ctx, 1, 0),
                        zs = coords(ctx, 2, 1);
    Field vx = host_field(ctx, SARAS_FIELD_VX), vy = host_field(ctx, SARAS_FIELD_VY);
    if (p.yInd == 0) {   // 2D (taylorGreen.cc:57-79): u and w on the y = 0 plane
        std::vector<double> zc = coords(ctx, 2, 0);
        Field vz = host_field(ctx, SARAS_FIELD_VZ);
        for (int i = -1; i < vx.dims[0] - 1; ++i)
            for (int k = -1; k < vx.dims[2] - 1; ++k)
                vx.at(i, 0, k) = std::sin(2.0 * M_PI * xc[i + 1] / L[0]) * std::cos(2.0 * M_PI * zs[k + 1] / L[2]);
        for (int i = -1; i < vz.dims[0] - 1; ++i)
            for (int k = -1; k < vz.dims[2] - 1; ++k)
                vz.at(i, 0, k) = -std::cos(2.0 * M_PI * xs[i + 1] / L[0]) * std::sin(2.0 * M_PI * zc[k + 1] / L[2]);
        check(saras_upload(ctx, SARAS_FIELD_VX, vx.v.data()), ctx, "upload Vx");
        check(saras_upload(ctx, SARAS_FIELD_VZ, vz.v.data()), ctx, "upload Vz");
        return;
    }
    for (int i = -1; i < vx.dims[0] - 1; ++i)
        for (int j = -1; j < vx.dims[1] - 1; ++j)
            for (int k = -1; k < vx.dims[2] - 1; ++k)
                vx.at(i, j, k) = std::sin(2.0 * M_PI * xc[i + 1] / L[0]) * std::cos(2.0 * M_PI * ys[j + 1] / L[1]) *
                                 std::cos(2.0 * M_PI * zs[k + 1] / L[2]);
    for (int i = -1; i < vy.dims[0] - 1; ++i)
        for (int j = -1; j < vy.dims[1] - 1; ++j)
            for (int k = -1; k < vy.dims[2] - 1; ++k)
                vy.at(i, j, k) = -std::cos(2.0 * M_PI * xs[i + 1] / L[0]) * std::sin(2.0 * M_PI * yc[j + 1] / L[1]) *
                                 std::cos(2.0 * M_PI * zs[k + 1] / L[2]);
    check(saras_upload(ctx, SARAS_FIELD_VX, vx.v.data()), ctx, "upload Vx");
    check(saras_upload(ctx, SARAS_FIELD_VY, vy.v.data()), ctx, "upload Vy");
}

}  // namespace

int main(int argc, char **argv) {
    const std::string input = argc > 1 ? argv[1] : "input/parameters.yaml";
    const std::string outdir = argc > 2 ? argv[2] : "output";
    struct timeval runStart, runEnd;
    saras_params p;
    char err[512] = {0};
    if (saras_parse_yaml(input.c_str(), &p, err, sizeof(err)) != SARAS_OK) abort_run(std::string("ERROR: ") + err);
    mkdir(outdir.c_str(), 0755);
    const bool scalar = p.probType >= 5;
    if (p.probType <= 0 || p.probType > 7) abort_run("Invalid problem type. ABORTING");
    static const char *kind[8] = {"", "lid-driven cavity problem", "decaying flow simulation", "channel flow problem",
                                  "forced channel flow problem", "heated bottom-plate problem", "heated top-plate problem",
                                  "heated sidewall problem"};
    std::cout << std::endl << "Solving NSE for " << kind[p.probType] << std::endl << std::endl;
    gettimeofday(&runStart, NULL);

    saras_ctx *ctx = nullptr;
    check(saras_create(&p, &ctx), nullptr, "creating the solver");
    // constructor (hydro_d3.cc:63-119, scalar_d3.cc:62-107)
    double time = 0.0;
    const std::string restartPath = outdir + "/restartFile.saras";
    if (p.restartFlag) {
        check(saras_read_restart(ctx, restartPath.c_str(), &time), ctx, "reading the restart file");
    } else {
        Field P = host_field(ctx, SARAS_FIELD_P);
        for (double &x : P.v) x = 1.0;
        check(saras_upload(ctx, SARAS_FIELD_P, P.v.data()), ctx, "upload P");
        if (!scalar) {
            if (p.icType == 1) {
                std::cout << "Imposing Taylor-Green vortices initial condition" << std::endl << std::endl;
                taylor_green(ctx, p);
            } else if (p.icType > 1) {
                abort_run("ERROR: channel-flow initial conditions are not available in this build");
            }
        }
    }
    const int nbc = scalar ? 4 : 3;
    const int bcf[4] = {SARAS_FIELD_VX, SARAS_FIELD_VY, SARAS_FIELD_VZ, SARAS_FIELD_T};
    for (int q = 0; q < nbc; ++q) check(saras_apply_bc(ctx, bcf[q]), ctx, "boundary conditions");

    // probes (probes.cc:61-98)
    std::vector<int> probes;
    std::ofstream probeFile;
    if (p.readProbes) {
        int n = 0;
        if (saras_parse_probes(input.c_str(), nullptr, 0, &n, err, sizeof(err)) != SARAS_OK) abort_run(std::string("ERROR: ") + err);
        probes.resize(3 * (size_t)n);
        if (saras_parse_probes(input.c_str(), probes.data(), n, &n, err, sizeof(err)) != SARAS_OK) abort_run(std::string("ERROR: ") + err);
        probeFile.open(outdir + "/ProbesData.dat", std::fstream::out | std::fstream::app);
        if (!p.restartFlag) probeFile << "#VARIABLES = Time, X, Y, Z, Vx, Vy, Vz, P" << (scalar ? ", T" : "") << std::endl;
    }
    const int pf[5] = {SARAS_FIELD_VX, SARAS_FIELD_VY, SARAS_FIELD_VZ, SARAS_FIELD_P, SARAS_FIELD_T};
    const int npf = scalar ? 5 : 4;
    auto probe_data = [&](double t) {   // probes::probeData (probes.cc:120-166)
        const int n = (int)(probes.size() / 3);
        std::vector<double> vals((size_t)n * npf);
        check(saras_probe(ctx, n, probes.data(), npf, pf, vals.data()), ctx, "probes");
        for (int q = 0; q < n; ++q) {
            probeFile << std::fixed << std::setw(6) << std::setprecision(4) << t << "\t" << std::setw(4) << std::setprecision(0)
                      << probes[3 * q] << "\t" << probes[3 * q + 1] << "\t" << probes[3 * q + 2] << "\t";
            probeFile << std::setw(16) << std::setprecision(8) << vals[(size_t)q * npf];
            for (int f = 1; f < npf; ++f) probeFile << "\t" << std::setw(16) << std::setprecision(8) << vals[(size_t)q * npf + f];
            probeFile << std::endl;
        }
    };

    // tseries (tseries.cc:62-124, 137-178, 195-246)
    std::ofstream ts(outdir + "/TimeSeries.dat", p.restartFlag ? std::fstream::app : std::fstream::out);
    double dt = p.tStp;
    check(saras_set_dt(ctx, dt), ctx, "time step");
    const double nu = scalar ? (p.rbcType == 1 ? p.Pr : p.rbcType == 3 ? 1.0 : std::sqrt(p.Pr / p.Ra)) : 0.0;
    if (!scalar) {
        std::cout << std::fixed << std::setw(6) << "Time" << "\t" << std::setw(16) << "Total energy" << "\t" << "Divergence" << std::endl;
        ts << "#VARIABLES = Time, Energy, Divergence, dt\n";
    } else {
        std::cout << std::fixed << std::setw(6) << "Time" << "\t" << std::setw(16) << "Re (Urms)" << "\t" << "Nusselt No" << "\t"
                  << "Divergence" << std::endl;
        ts << "#VARIABLES = Time, Energy, NusseltNo, Divergence, dt\n";
    }
    auto write_ts = [&]() {
        double e = 0, d = 0, nuNo = 0;
        check(saras_diagnostics(ctx, &e, &d, &nuNo), ctx, "time series");
        if (!scalar) {
            std::cout << std::fixed << std::setw(6) << std::setprecision(4) << time << "\t" << std::setw(16) << std::setprecision(8) << e
                      << "\t" << d << std::endl;
            ts << std::fixed << std::setw(6) << std::setprecision(4) << time << "\t" << std::setw(16) << std::setprecision(8) << e << "\t"
               << d << "\t" << dt << std::endl;
        } else {
            std::cout << std::fixed << std::setw(6) << std::setprecision(4) << time << "\t" << std::setw(16) << std::setprecision(8)
                      << std::sqrt(e) / nu << "\t" << nuNo << "\t" << d << std::endl;
            ts << std::fixed << std::setw(6) << std::setprecision(4) << time << "\t" << std::setw(16) << std::setprecision(8)
               << std::sqrt(e) / nu << "\t" << nuNo << "\t" << d << "\t" << dt << std::endl;
        }
    };

    // solvePDE (hydro_d3.cc:122-251)
    write_ts();
    if (!p.restartFlag && p.readProbes) probe_data(time);
    double prTime = time + p.prInt - std::fmod(time, p.prInt);
    double rsTime = time + p.rsInt - std::fmod(time, p.rsInt);
    long timeStepCount = 0;
    while (true) {
        saras_step_stats st;
        check(saras_time_advance(ctx, &st), ctx, "time step");
        if (p.useCFL) {
            check(saras_compute_tstp(ctx, &dt), ctx, "CFL time step");
            if (dt > p.tStp) dt = p.tStp;
            check(saras_set_dt(ctx, dt), ctx, "time step");
        }
        timeStepCount += 1;
        time += dt;
        if (timeStepCount % std::max(1, p.ioCnt) == 0) write_ts();
        if (p.readProbes && std::abs(prTime - time) < 0.5 * dt) {
            probe_data(time);
            prTime += p.prInt;
        }
        if (std::abs(rsTime - time) < 0.5 * dt) {
            check(saras_write_restart(ctx, restartPath.c_str(), time), ctx, "writing the restart file");
            rsTime += p.rsInt;
        }
        if (std::abs(p.tMax - time) < 0.5 * dt) break;
    }
    saras_destroy(ctx);
    gettimeofday(&runEnd, NULL);
    double run_time = ((runEnd.tv_sec - runStart.tv_sec) * 1000000u + runEnd.tv_usec - runStart.tv_usec) / 1.e6;
    std::cout << std::endl << "Simulation completed" << std::endl << std::endl;
    std::cout << "Time taken by simulation: " << run_time << std::endl;
    return 0;
}
