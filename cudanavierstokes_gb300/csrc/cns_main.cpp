// cns_main.cpp -- drop-in driver with the reference executable's behaviour
// (src/main.cpp:22-79, src/cuda_main.cu:267-324, src/init.cpp), on the C ABI.
//
//   cns <parameter file> [run directory]
//
// The parameter file holds "name = value" lines with the reference's globals.h names
// (mx_tot, my_tot, mz_tot, Lx, Ly, Lz, stencilSize, stencilVisc, nsteps, nfiles, CFL,
// restartFile, lowStorage, boundaryLayer, perturbed, forcing, periodicX, nonUniformX,
// checkCFLcondition, checkBulk, Re, Pr, Ma, viscexp, gam, stretch, TwallTop, TwallBot) plus
// optional precision (0 FP64, 1 FP32 RHS, 2 FP32-pair RHS) and quirk_dissipation_y. Output as the reference:
// fields/{x,y,z}.bin, Grid.txt, fields/{r,u,v,w,e}.%07d.bin (raw FP64, [k][j][i]),
// solution.txt ("step time kin par2 dtime" every checkCFLcondition steps), prof.txt (plane
// profiles, after each file) and the printed friction Reynolds number, and an XDMF
// descriptor fields/fields.xmf of the files this run wrote. A boundary layer
// reads blasius1D/{x,r,u,w,e}Prof.bin. Without restart the initial field is the reference's
// own: initChannel (forcing), initCHIT (periodic box) or the sponge reference fields.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cns.h"

namespace {

std::map<std::string, std::string> read_kv(const char* path) {
    std::map<std::string, std::string> kv;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        auto trim = [](std::string s) {
            const size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
            return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
        };
        kv[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
    }
    return kv;
}

bool as_bool(const std::string& v) { return v == "1" || v == "true" || v == "(true)" || v == "True"; }

bool write_bin(const std::string& path, const double* a, size_t n) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = fwrite(a, sizeof(double), n, f) == n;
    fclose(f);
    return ok;
}

bool read_bin(const std::string& path, std::vector<double>& a) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    const long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    a.resize(bytes / sizeof(double));
    const bool ok = fread(a.data(), sizeof(double), a.size(), f) == a.size();
    fclose(f);
    return ok;
}

// XDMF 2 descriptor of the written fields (the format python-utils/writexmf.py produces
// for the reference's output): a 3D rectilinear mesh from x, y, z and a temporal
// collection with one uniform grid per file index, its r, u, v, w, e attributes read as
// native-endian FP64 binaries from fields/%c.%07d.bin.
bool write_xmf(const std::string& path, const std::vector<double>& x, const std::vector<double>& y,
               const std::vector<double>& z, const std::vector<std::pair<int, double>>& files) {
    FILE* f = fopen(path.c_str(), "w");
    if (!f) return false;
    const char* xml = "Format=\"XML\" DataType=\"Float\" Precision=\"8\"";
    const char* bin = "Format=\"Binary\" DataType=\"Float\" Precision=\"8\" Endian=\"Native\"";
    const size_t nx = x.size(), ny = y.size(), nz = z.size();
    fprintf(f, "<?xml version=\"1.0\" ?>\n<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n");
    fprintf(f, "<Xdmf xmlns:xi=\"http://www.w3.org/2001/XInclude\" Version=\"2.0\">\n<Domain>\n");
    fprintf(f, "    <Topology name=\"TOPO\" TopologyType=\"3DRectMesh\" Dimensions=\"%zu %zu %zu\"/>\n", nz, ny, nx);
    fprintf(f, "    <Geometry name=\"GEO\" GeometryType=\"VXVYVZ\">\n");
    for (const auto* a : {&x, &y, &z}) {
        fprintf(f, "        <DataItem %s Dimensions=\"%zu\">\n", xml, a->size());
        for (double v : *a) fprintf(f, " %.15e", v);
        fprintf(f, "\n        </DataItem>\n");
    }
    fprintf(f, "    </Geometry>\n");
    fprintf(f, "    <Grid Name=\"TimeSeries\" GridType=\"Collection\" CollectionType=\"Temporal\">\n");
    fprintf(f, "        <Time TimeType=\"List\">\n            <DataItem %s Dimensions=\"%zu\">\n", xml, files.size());
    for (const auto& t : files) fprintf(f, " %.15e", t.second);
    fprintf(f, "\n            </DataItem>\n        </Time>\n");
    for (const auto& t : files) {
        fprintf(f, "        <Grid Name=\"T%07d\" GridType=\"Uniform\">\n", t.first);
        fprintf(f, "            <Topology Reference=\"/Xdmf/Domain/Topology[1]\"/>\n");
        fprintf(f, "            <Geometry Reference=\"/Xdmf/Domain/Geometry[1]\"/>\n");
        for (const char* n : {"r", "u", "v", "w", "e"}) {
            fprintf(f, "            <Attribute Name=\"%s\" Center=\"Node\">\n", n);
            fprintf(f, "                <DataItem %s Dimensions=\"%zu %zu %zu\">\n", bin, nz, ny, nx);
            fprintf(f, "                    %s.%07d.bin\n                </DataItem>\n            </Attribute>\n", n,
                    t.first);
        }
        fprintf(f, "        </Grid>\n");
    }
    fprintf(f, "    </Grid>\n</Domain>\n</Xdmf>\n");
    return fclose(f) == 0;
}

// time, dt and body force beside each field file, so a restart continues the clock and
// the forcing controller (the reference restarts both from their initial values)
std::string scalars_name(const std::string& dir, int step) {
    char buf[64];
    snprintf(buf, sizeof buf, "/fields/scalars.%07d.txt", step);
    return dir + buf;
}

void write_scalars(cns_solver* h, const std::string& dir, int step) {
    double dt = 0, dpdz = 0, t = 0;
    cns_get_scalars(h, &dt, &dpdz, &t);
    if (FILE* f = fopen(scalars_name(dir, step).c_str(), "w")) {
        fprintf(f, "time = %.17g\ndt = %.17g\ndpdz = %.17g\n", t, dt, dpdz);
        fclose(f);
    }
}

// calcAvgChan's prof.txt (src/init.cpp:150-208) from the device plane statistics
void write_prof(cns_solver* h, const std::string& dir, int mx) {
    std::vector<double> st(11 * (size_t)mx);
    if (cns_plane_stats(h, st.data()) != CNS_OK) return;
    if (FILE* f = fopen((dir + "/prof.txt").c_str(), "w")) {
        for (int i = 0; i < mx; i++) {
            for (int q = 0; q < 11; q++) fprintf(f, q ? "\t%lf" : "%lf", st[(size_t)q * mx + i]);
            fprintf(f, "\n");
        }
        fclose(f);
    }
}

std::string field_name(const std::string& dir, char c, int step) {
    char buf[64];
    snprintf(buf, sizeof buf, "/fields/%c.%07d.bin", c, step);
    return dir + buf;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <parameter file> [run directory]\n", argv[0]);
        return 1;
    }
    const std::string dir = argc > 2 ? argv[2] : ".";
    auto kv = read_kv(argv[1]);
    cns_params p;
    cns_default_params(&p);
    auto geti = [&](const char* k, int d) { return kv.count(k) ? (int)std::strtol(kv[k].c_str(), nullptr, 0) : d; };
    auto getd = [&](const char* k, double d) { return kv.count(k) ? std::strtod(kv[k].c_str(), nullptr) : d; };
    auto getb = [&](const char* k, bool d) { return kv.count(k) ? as_bool(kv[k]) : d; };
    p.mx = geti("mx_tot", p.mx); p.my = geti("my_tot", p.my); p.mz = geti("mz_tot", p.mz);
    p.Lx = getd("Lx", p.Lx); p.Ly = getd("Ly", p.Ly); p.Lz = getd("Lz", p.Lz);
    p.stencil_size = geti("stencilSize", p.stencil_size);
    p.stencil_visc = geti("stencilVisc", p.stencil_visc);
    p.cfl = getd("CFL", p.cfl);
    p.scheme = getb("lowStorage", true) ? CNS_RK3_LOWSTORAGE : CNS_RK3_CLASSIC;
    p.boundary_layer = getb("boundaryLayer", false);
    p.perturbed = getb("perturbed", false);
    p.forcing = getb("forcing", false);
    p.periodic_x = getb("periodicX", true);
    p.nonuniform_x = getb("nonUniformX", false);
    p.check_cfl = geti("checkCFLcondition", p.check_cfl);
    p.check_bulk = geti("checkBulk", p.check_bulk);
    p.Re = getd("Re", p.Re); p.Pr = getd("Pr", p.Pr); p.Ma = getd("Ma", p.Ma);
    p.viscexp = getd("viscexp", p.viscexp); p.gam = getd("gam", p.gam);
    p.stretch = getd("stretch", p.stretch);
    p.twall_top = getd("TwallTop", p.twall_top); p.twall_bot = getd("TwallBot", p.twall_bot);
    p.precision = geti("precision", CNS_PREC_FP64);
    p.quirk_dissipation_y = geti("quirk_dissipation_y", 1);
    const int nsteps = geti("nsteps", 100), nfiles = geti("nfiles", 1), restart = geti("restartFile", -1);
    const int device = geti("device", 0);
    if (cns_check_params(&p) != CNS_OK) {
        fprintf(stderr, "invalid parameters: %s\n", cns_last_error());
        return 1;
    }
    const auto t_begin = std::chrono::steady_clock::now();
    const size_t N = (size_t)p.mx * p.my * p.mz;

    // initGrid (src/init.cpp:32-92): grid files before any device work
    std::vector<double> x(p.mx), xp(p.mx), xpp(p.mx), y(p.my), z(p.mz);
    cns_host_grid(&p, x.data(), xp.data(), xpp.data(), y.data(), z.data());
    std::string mk = "mkdir -p '" + dir + "/fields'";
    if (system(mk.c_str()) != 0) fprintf(stderr, "warning: could not create %s/fields\n", dir.c_str());
    write_bin(dir + "/fields/x.bin", x.data(), x.size());
    write_bin(dir + "/fields/y.bin", y.data(), y.size());
    write_bin(dir + "/fields/z.bin", z.data(), z.size());
    if (FILE* g = fopen((dir + "/Grid.txt").c_str(), "w")) {
        for (int i = 0; i < p.mx; i++) fprintf(g, "%d %lf %lf %lf\n", i, x[i], xp[i], xpp[i]);
        fclose(g);
    }

    cns_solver* h = nullptr;
    if (cns_create(&p, device, &h) != CNS_OK) {
        fprintf(stderr, "cns_create: %s\n", cns_last_error());
        return 2;
    }
    std::vector<double> f[5];
    for (auto& a : f) a.assign(N, 0.0);
    bool have_fields = false;
    if (p.boundary_layer) {
        // calculateSponge (src/sponge.cu:83-240) from blasius1D/*Prof.bin
        std::vector<double> prof[5];
        const char* names = "xruwe";
        for (int q = 0; q < 5; q++)
            if (!read_bin(dir + "/blasius1D/" + names[q] + "Prof.bin", prof[q])) {
                fprintf(stderr, "cannot read %s/blasius1D/%cProf.bin\n", dir.c_str(), names[q]);
                cns_destroy(h);
                return 3;
            }
        if (cns_set_sponge_profiles(h, (int)prof[0].size(), prof[0].data(), prof[1].data(), prof[2].data(),
                                    prof[3].data(), prof[4].data(), restart < 0) != CNS_OK) {
            fprintf(stderr, "sponge: %s\n", cns_last_error());
            cns_destroy(h);
            return 3;
        }
        have_fields = restart < 0;
    }
    const double Rgas = 1.0 / (p.gam * p.Ma * p.Ma);
    if (restart >= 0) {
        // initField (src/init.cpp:13-22)
        const char* names = "ruvwe";
        for (int q = 0; q < 5; q++) {
            std::vector<double> a;
            if (!read_bin(field_name(dir, names[q], restart), a) || a.size() != N) {
                fprintf(stderr, "cannot read restart field %s\n", field_name(dir, names[q], restart).c_str());
                cns_destroy(h);
                return 3;
            }
            f[q] = a;
        }
    } else if (p.forcing) {
        // initChannel (src/init.cpp:94-124)
        const double U0 = std::pow(p.gam, 0.5) * p.Ma, P0 = 1.0 * Rgas, R0 = 1.0;
        for (int i = 0; i < p.mx; i++)
            for (int j = 0; j < p.my; j++)
                for (int k = 0; k < p.mz; k++) {
                    const size_t c = (size_t)i + (size_t)j * p.mx + (size_t)k * p.mx * p.my;
                    double rr1 = rand() * 1.0 / (RAND_MAX * 1.0) - 0.5;
                    double rr2 = rand() * 1.0 / (RAND_MAX * 1.0) - 0.5;
                    double rr3 = rand() * 1.0 / (RAND_MAX * 1.0) - 0.5;
                    double uf = 0.02 * rr1 + 0.05 * sin(0.5 * M_PI * x[i]) * cos(2 * M_PI * y[j]);
                    double vf = 0.02 * rr2 + 0.05 * sin(0.5 * M_PI * x[i]) * sin(2 * M_PI * y[j]);
                    double wf = 0.02 * rr3;
                    const double wmean = 1.5 * U0 * R0 * x[i] * (1.0 - x[i] / p.Lx);
                    f[1][c] = uf; f[2][c] = vf; f[3][c] = wmean + wf; f[0][c] = R0;
                    f[4][c] = P0 / (p.gam - 1.0) + 0.5 * R0 * (uf * uf + vf * vf + f[3][c] * f[3][c]);
                }
    } else if (!p.boundary_layer) {
        // initCHIT (src/init.cpp:126-148)
        const double V0 = 1.0, T0 = 1.0, P0 = T0 * Rgas, R0 = 1.0;
        for (int i = 0; i < p.mx; i++)
            for (int j = 0; j < p.my; j++)
                for (int k = 0; k < p.mz; k++) {
                    const double fx = 2 * M_PI * x[i] / p.Lx, fy = 2 * M_PI * y[j] / p.Ly, fz = 2 * M_PI * z[k] / p.Lz;
                    const size_t c = (size_t)i + (size_t)j * p.mx + (size_t)k * p.mx * p.my;
                    f[1][c] = V0 * sin(fx) * cos(fy) * cos(fz);
                    f[2][c] = -V0 * cos(fx) * sin(fy) * cos(fz);
                    f[3][c] = 0.0;
                    const double press = P0 + 1.0 / 16.0 * R0 * V0 * V0 * (cos(2.0 * fx) + cos(2.0 * fy)) * (cos(2.0 * fz) + 2.0);
                    f[0][c] = press / Rgas / T0;
                    f[4][c] = press / (p.gam - 1.0) +
                              0.5 * f[0][c] * (f[1][c] * f[1][c] + f[2][c] * f[2][c] + f[3][c] * f[3][c]);
                }
    }
    if (!have_fields) {
        if (cns_copy_field(h, 0, f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data()) != CNS_OK) {
            fprintf(stderr, "copy in: %s\n", cns_last_error());
            cns_destroy(h);
            return 2;
        }
    }
    if (restart >= 0) {
        auto sc = read_kv(scalars_name(dir, restart).c_str());
        if (sc.count("time") && sc.count("dt") && sc.count("dpdz"))
            cns_set_scalars(h, std::strtod(sc["dt"].c_str(), nullptr), std::strtod(sc["dpdz"].c_str(), nullptr),
                            std::strtod(sc["time"].c_str(), nullptr), -1);
    }
    // printRes and calcAvgChan of the initial field (src/main.cpp:58-59)
    double ret = 0;
    if (cns_friction_reynolds(h, &ret) == CNS_OK) printf("\nThe average friction Reynolds number is: \t %lf\n", ret);
    write_prof(h, dir, p.mx);
    std::vector<std::pair<int, double>> written;
    {
        double t0 = 0;
        cns_get_scalars(h, nullptr, nullptr, &t0);
        written.push_back({restart < 0 ? 0 : restart, t0});
    }
    if (restart < 0) {
        cns_copy_field(h, 1, f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data());
        const char* names = "ruvwe";
        for (int q = 0; q < 5; q++) write_bin(field_name(dir, names[q], 0), f[q].data(), N);
        write_scalars(h, dir, 0);
    }

    // solverWrapper (src/cuda_main.cu:267-324)
    const int start = restart < 0 ? 0 : restart;
    FILE* sol = fopen((dir + "/solution.txt").c_str(), "w");
    std::vector<double> par1(nsteps), par2(nsteps), tim(nsteps);
    double tprev = 0.0;
    int rc = CNS_OK;
    for (int file = start + 1; file < nfiles + start + 1 && rc == CNS_OK; file++) {
        rc = cns_run(h, nsteps, par1.data(), par2.data(), tim.data());
        if (rc != CNS_OK) {
            fprintf(stderr, "cns_run: %s\n", cns_last_error());
            break;
        }
        cns_copy_field(h, 1, f[0].data(), f[1].data(), f[2].data(), f[3].data(), f[4].data());
        const char* names = "ruvwe";
        for (int q = 0; q < 5; q++) write_bin(field_name(dir, names[q], file), f[q].data(), N);
        write_scalars(h, dir, file);
        written.push_back({file, tim[nsteps - 1]});
        write_prof(h, dir, p.mx);   // calcAvgChan after each file (src/cuda_main.cu:311)
        printf("file number: %d  \t step: %d  \t time: %lf  \t kin: %le  \t energy: %le\n", file, file * nsteps,
               tim[nsteps - 1], par1[0], par2[0]);
        if (sol)
            for (int t = 0; t < nsteps - 1; t += p.check_cfl)
                fprintf(sol, "%d %lf %lf %lf %lf\n", file * (t + 1), tim[t], par1[t], par2[t],
                        (t + 1 < nsteps ? tim[t + 1] : tim[t]) - tim[t]);
        tprev = tim[nsteps - 1];
    }
    if (sol) fclose(sol);
    write_xmf(dir + "/fields/fields.xmf", x, y, z, written);
    cns_destroy(h);
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_begin).count();
    printf("The total time is: %g\n", total);
    printf("The simulation time per time step is: %g\n", total / ((double)nfiles * nsteps));
    printf("Simulation is finished! (t = %g)\n", tprev);
    return rc == CNS_OK ? 0 : 4;
}
