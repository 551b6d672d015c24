// poe2d_cli.cpp -- drop-in driver for the reference program's main()
// (seismic_CPML_2D_poroelastic_withCUDA.cu, cited cu:).
//
// Reads what the reference reads and writes what it writes, in its formats:
//   input1.txt   NSTEP ISOURCE JSOURCE a0_pos a1_pos     (cu:500, 757-762)
//   input2.txt   f0                                     (cu:830)
//   model files  medium-ID, cp, cs, saturated-density grids, raw float32,
//                (NX+1)(NZ+1) values x fastest (cu:606-644); --order z reads
//                the z-fastest files patchymodel.m writes (patchy:50-51)
//   mediumrho.ctxt          cp grid, float32 x fastest  (cu:1476-1487)
//   vz%05i.vzo / vx%05i.vxo snapshots every samp steps  (cu:1653-1727)
//   recvspvz/recvspvx%08i.vsp, rechorvz/rechorvx%08i.hor: one text row per
//                step, values followed by a space        (cu:1742-1872)
//   recats/recbwh/recsrc%08i.ats/.bwh/.src: one text line of NSTEP values
//                ("%08f" names when f0 < 1)              (cu:1875-1905)
// Text goes through std::ofstream with default formatting, exactly as the
// reference prints its floats.
//
// The reference's hard-coded constants are the defaults; flags override
// them.  Differences: every one of the NSTEP steps is run, where the
// reference runs NSTEP/samp*samp of them (cu:1620) and leaves the trace rows
// after those zero (cu:1251-1305 clear them, cu:1737-1905 write all NSTEP
// rows); --ref-steps runs the reference's count and writes those zero rows.
// Errors exit non-zero with a message (the reference crashed on a missing
// model file), and a Courant failure prints the reference's message and
// returns 0 as the reference does (cu:1200-1212).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "poe2d.h"

namespace {

struct Opts {
    int nx = 13599, nz = 2439;             // cu:486-487
    float dx = 1.25f, dt = 95e-06f;        // cu:493, 506
    int panj = 122, panj2 = 680;           // cu:496-497
    int samp = 5000;                       // cu:501
    int npml = 10;                         // cu:513
    std::string in_dir = ".", out_dir = ".";
    std::string medium = "mar_poro_2440x13600.bin", cp = "mar_cp_2440x13600.bin";   // cu:606, 616
    std::string cs = "mar_cs_2440x13600.bin", rho = "mar_rho_2440x13600.bin";       // cu:626, 636
    std::string fluid;                     // optional table file: rows of K_f eta kappa phi tortuosity rho_f
    std::string checkpoint, restart;       // full-state image written at each snapshot / read at start
    char order = 'x';
    bool fast = false, dry = false, snapshots = true, medium_dump = true;
    bool ref_steps = false;                // run NSTEP/samp*samp steps, as the reference's loop does
};

// the reference's fluid table, medium IDs 0..3 (cu:565-568, 574-575)
const float kRefFluid[4][6] = {
    {2.4e09f, 0.003f, 1.5e-17f, 1.e-6f, 2.0f, 10.0f},
    {2.4e09f, 0.003f, 500.0e-15f, 1.e-6f, 2.0f, 10.0f},
    {0.7e09f, 0.03f, 500.0e-15f, 1.e-6f, 2.0f, 10.0f},
    {0.02e09f, 1.0e-5f, 500.0e-15f, 1.e-6f, 2.0f, 10.0f},
};

void usage()
{
    std::cerr <<
        "poe2d_run [options]   drop-in for the reference's main()\n"
        "  --nx N --nz N          grid is (NX+1) x (NZ+1)            [13599 2439]\n"
        "  --dx H --dt S          cell size (m), time step (s)        [1.25 9.5e-05]\n"
        "  --panj N --panj2 N     VSP / horizontal receiver counts    [122 680]\n"
        "  --samp N               snapshot interval in steps          [5000]\n"
        "  --npml N               C-PML thickness in cells            [10]\n"
        "  --medium F --cp F --cs F --rho F   model files (float32)\n"
        "  --order x|z            x fastest (arr2bin) or z fastest (patchymodel.m)  [x]\n"
        "  --fluid F              fluid table, one row per medium ID: K_f eta kappa phi tortuosity rho_f\n"
        "  --in DIR --out DIR     where input1.txt/input2.txt/models are, where outputs go  [. .]\n"
        "  --fast                 plain FP32 stencils (default: the reference's rounding)\n"
        "  --no-snapshots         skip the .vzo/.vxo files\n"
        "  --no-medium-dump       skip mediumrho.ctxt\n"
        "  --checkpoint F         write the shot's full state to F at every snapshot (restartable)\n"
        "  --restart F            continue from a --checkpoint image of the same run\n"
        "  --ref-steps            run NSTEP/samp*samp steps as the reference does; later trace rows are 0\n"
        "  --dry-run              read and check inputs, build coefficients and profiles, no GPU\n";
}

bool parse(int argc, char **argv, Opts &o)
{
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto val = [&](const char *name) -> const char * {
            if (i + 1 >= argc) {
                std::cerr << "missing value for " << name << "\n";
                return nullptr;
            }
            return argv[++i];
        };
        const char *v = nullptr;
#define INT_OPT(flag, field) \
    else if (a == flag) { if (!(v = val(flag))) return false; o.field = std::atoi(v); }
#define FLT_OPT(flag, field) \
    else if (a == flag) { if (!(v = val(flag))) return false; o.field = (float)std::atof(v); }
#define STR_OPT(flag, field) \
    else if (a == flag) { if (!(v = val(flag))) return false; o.field = v; }
        if (a == "-h" || a == "--help") { usage(); std::exit(0); }
        INT_OPT("--nx", nx) INT_OPT("--nz", nz) FLT_OPT("--dx", dx) FLT_OPT("--dt", dt)
        INT_OPT("--panj", panj) INT_OPT("--panj2", panj2) INT_OPT("--samp", samp) INT_OPT("--npml", npml)
        STR_OPT("--medium", medium) STR_OPT("--cp", cp) STR_OPT("--cs", cs) STR_OPT("--rho", rho)
        STR_OPT("--fluid", fluid) STR_OPT("--in", in_dir) STR_OPT("--out", out_dir)
        STR_OPT("--checkpoint", checkpoint) STR_OPT("--restart", restart)
        else if (a == "--order") {
            if (!(v = val("--order"))) return false;
            o.order = v[0];
            if ((o.order != 'x' && o.order != 'z') || v[1]) { std::cerr << "--order x|z\n"; return false; }
        }
        else if (a == "--fast") o.fast = true;
        else if (a == "--dry-run") o.dry = true;
        else if (a == "--no-snapshots") o.snapshots = false;
        else if (a == "--no-medium-dump") o.medium_dump = false;
        else if (a == "--ref-steps") o.ref_steps = true;
        else { std::cerr << "unknown option " << a << "\n"; usage(); return false; }
#undef INT_OPT
#undef FLT_OPT
#undef STR_OPT
    }
    if (o.nx < 4 || o.nz < 4 || o.samp < 1 || o.panj < 1 || o.panj2 < 1 || o.npml < 1 || !(o.dx > 0) || !(o.dt > 0)) {
        std::cerr << "invalid grid, time or receiver parameters\n";
        return false;
    }
    return true;
}

std::string path(const std::string &dir, const std::string &f)
{
    if (f.empty() || f[0] == '/' || dir.empty() || dir == ".") return f;
    return dir + "/" + f;
}

// (NX+1)(NZ+1) float32 values, returned x fastest
bool read_grid(const std::string &file, int nx1, int nz1, char order, std::vector<float> &out)
{
    std::FILE *f = std::fopen(file.c_str(), "rb");
    if (!f) {
        std::cerr << file << ": cannot open\n";
        return false;
    }
    const size_t n = (size_t)nx1 * nz1;
    std::vector<float> raw(n);
    const size_t got = std::fread(raw.data(), sizeof(float), n, f);
    std::fclose(f);
    if (got != n) {
        std::cerr << file << ": " << got << " floats, expected " << n << "\n";
        return false;
    }
    if (order == 'x') {
        out.swap(raw);
    } else {   // z fastest: raw[x * nz1 + z]
        out.resize(n);
        for (int x = 0; x < nx1; ++x)
            for (int z = 0; z < nz1; ++z) out[(size_t)z * nx1 + x] = raw[(size_t)x * nz1 + z];
    }
    return true;
}

bool read_fluid(const std::string &file, std::vector<float> &tab)
{
    tab.clear();
    if (file.empty()) {
        for (const auto &r : kRefFluid) tab.insert(tab.end(), r, r + 6);
        return true;
    }
    std::ifstream in(file);
    if (!in.is_open()) {
        std::cerr << file << ": cannot open\n";
        return false;
    }
    float v;
    while (in >> v) tab.push_back(v);
    if (tab.empty() || tab.size() % 6) {
        std::cerr << file << ": expected rows of 6 values\n";
        return false;
    }
    return true;
}

bool write_raw(const std::string &file, const float *v, size_t n)
{
    std::FILE *f = std::fopen(file.c_str(), "wb");
    if (!f) {
        std::cerr << file << ": cannot write\n";
        return false;
    }
    const bool ok = std::fwrite(v, sizeof(float), n, f) == n;
    std::fclose(f);
    return ok;
}

// rows of `cols` values, "v " each, "\n" after a row (cu:1772-1781)
bool write_rows(const std::string &file, const std::vector<float> &tr, int64_t rows, int nrec, int col0, int cols)
{
    std::ofstream out(file);
    if (!out.is_open()) return false;
    for (int64_t r = 0; r < rows; ++r) {
        const float *row = tr.data() + r * nrec + col0;
        for (int c = 0; c < cols; ++c) out << row[c] << " ";
        out << "\n";
    }
    return (bool)out;
}

// one line of values, "v " each (cu:1893-1905)
bool write_line(const std::string &file, const std::vector<float> &tr, int64_t rows, int nrec, int col)
{
    std::ofstream out(file);
    if (!out.is_open()) return false;
    for (int64_t r = 0; r < rows; ++r) out << tr[r * nrec + col] << " ";
    return (bool)out;
}

int fail(poe_ctx *ctx, int st, const char *what)
{
    std::cerr << what << ": " << poe_status_string(st);
    if (ctx) std::cerr << " (" << poe_last_error(ctx) << ")";
    std::cerr << "\n";
    if (ctx) poe_destroy(ctx);
    return 1;
}

}  // namespace

int main(int argc, char **argv)
{
    Opts o;
    if (!parse(argc, argv, o)) return 2;
    std::ifstream in1(path(o.in_dir, "input1.txt"));
    if (!in1.is_open()) {
        std::printf("File not opened...");   // cu:473-477
        return 1;
    }
    std::ifstream in2(path(o.in_dir, "input2.txt"));
    if (!in2.is_open()) {
        std::printf("File not opened...");   // cu:480-484
        return 1;
    }
    int64_t nstep = 0;
    int isrc = 0, jsrc = 0, a0 = 0, a1 = 0;
    float f0 = 0.0f;
    if (!(in1 >> nstep >> isrc >> jsrc >> a0 >> a1) || !(in2 >> f0)) {
        std::cerr << "input1.txt needs NSTEP ISOURCE JSOURCE a0_pos a1_pos, input2.txt needs f0\n";
        return 1;
    }
    if (nstep < 1 || !(f0 > 0.0f)) {
        std::cerr << "NSTEP must be positive and f0 > 0\n";
        return 1;
    }
    const int nx1 = o.nx + 1, nz1 = o.nz + 1;
    const size_t n = (size_t)nx1 * nz1;
    std::vector<float> medium, cp, cs, rho, fluid;
    if (!read_grid(path(o.in_dir, o.medium), nx1, nz1, o.order, medium) ||
        !read_grid(path(o.in_dir, o.cp), nx1, nz1, o.order, cp) ||
        !read_grid(path(o.in_dir, o.cs), nx1, nz1, o.order, cs) ||
        !read_grid(path(o.in_dir, o.rho), nx1, nz1, o.order, rho) || !read_fluid(o.fluid, fluid))
        return 1;

    poe_grid g = {o.nx, o.nz, o.dx, o.dx, o.dt};   // DELTAZ = DELTAX (cu:494)
    std::vector<float> coef(8 * n), px(6 * (size_t)nx1), pz(6 * (size_t)nz1);
    int st = poe_coeffs_from_medium(&g, medium.data(), cp.data(), cs.data(), rho.data(), fluid.data(),
                                    (int32_t)(fluid.size() / 6), coef.data());
    if (st != POE_OK) return fail(nullptr, st, "medium (IDs must index the fluid table)");
    float cpmax = 0.0f;
    for (float v : cp) cpmax = std::fmax(cpmax, v);
    poe_pml_params pml;
    poe_pml_defaults(&pml, o.npml, f0, cpmax);
    if ((st = poe_pml_build(&g, &pml, px.data(), pz.data())) != POE_OK) return fail(nullptr, st, "C-PML profiles");
    if (poe_check_courant(&g, cpmax) != POE_OK) {
        std::cout << "'time step is too large, simulation will be unstable'";   // cu:1200-1212
        return 0;
    }
    if (isrc < 0 || isrc > o.nx || jsrc < 0 || jsrc > o.nz) {
        std::cerr << "source (" << isrc << ", " << jsrc << ") outside the grid\n";
        return 1;
    }
    const int ncap = 2 * o.panj + 2 * o.panj2 + 4;
    std::vector<poe_receiver> rec((size_t)ncap);
    const int nrec = poe_ref_receivers(&g, isrc, jsrc, o.panj, o.panj2, a0, a1, rec.data(), ncap);
    if (nrec != ncap) {
        std::cerr << "receiver geometry\n";
        return 1;
    }
    if (o.medium_dump && !write_raw(path(o.out_dir, "mediumrho.ctxt"), cp.data(), n)) return 1;
    // steps the loop runs: all of them, or the reference's whole chunks (cu:1620)
    const int64_t nrun = o.ref_steps ? nstep / o.samp * o.samp : nstep;
    std::cout << "grid " << nx1 << " x " << nz1 << ", NSTEP=" << nstep << ", source (" << isrc << ", " << jsrc
              << "), f0=" << f0 << ", " << nrec << " receivers, " << nrun << " steps run\n";
    if (o.dry) return 0;
    medium.clear();
    cs.clear();
    rho.clear();

    poe_ctx *ctx = nullptr;
    if ((st = poe_create(&g, coef.data(), px.data(), pz.data(), nullptr, o.fast ? POE_CTX_FAST_STENCIL : 0, &ctx)) !=
        POE_OK)
        return fail(ctx, st, "create");
    coef.clear();
    const poe_source src = {isrc, jsrc, POE_SRC_REF_DGAUSS_P, f0, 1.0f, 0.4};   // cu:90-111
    int32_t shot = 0;
    if ((st = poe_add_shot(ctx, &src, rec.data(), nrec, &shot)) != POE_OK) return fail(ctx, st, "shot");

    int64_t done = 0;
    if (!o.restart.empty()) {   // continue where a checkpointed run stopped
        std::FILE *f = std::fopen(o.restart.c_str(), "rb");
        if (!f) return fail(ctx, POE_EIO, o.restart.c_str());
        std::vector<char> img;
        char chunk[1 << 16];
        size_t got;
        while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) img.insert(img.end(), chunk, chunk + got);
        std::fclose(f);
        if ((st = poe_checkpoint_load(ctx, shot, img.data(), (int64_t)img.size())) != POE_OK)
            return fail(ctx, st, "restart");
        poe_steps_done(ctx, shot, &done);
        if (done > nrun) return fail(ctx, POE_EINVAL, "checkpoint is past the steps to run");
    }
    std::vector<float> snap(o.snapshots ? n : 0);
    char name[128];
    while (done < nrun) {   // chunks of samp steps with their snapshots (cu:1620-1727)
        const int64_t k = std::min<int64_t>(o.samp - done % o.samp, nrun - done);
        if ((st = poe_run(ctx, k)) != POE_OK) return fail(ctx, st, "run");
        done += k;
        if (done % o.samp == 0 && !o.checkpoint.empty()) {
            int64_t bytes = 0;
            poe_checkpoint_size(ctx, shot, &bytes);
            std::vector<char> img((size_t)bytes);
            if ((st = poe_checkpoint_save(ctx, shot, img.data(), bytes)) != POE_OK) return fail(ctx, st, "checkpoint");
            const std::string tmp = o.checkpoint + ".tmp";
            std::FILE *f = std::fopen(tmp.c_str(), "wb");
            const bool w = f && std::fwrite(img.data(), 1, img.size(), f) == img.size();
            if (f) std::fclose(f);
            if (!w || std::rename(tmp.c_str(), o.checkpoint.c_str()) != 0) return fail(ctx, POE_EIO, "checkpoint file");
        }
        if (done % o.samp == 0 && o.snapshots) {
            std::snprintf(name, sizeof name, "vz%05i.vzo", (int)done);
            if ((st = poe_get_field(ctx, shot, POE_F_VZ, snap.data())) != POE_OK) return fail(ctx, st, "vz");
            if (!write_raw(path(o.out_dir, name), snap.data(), n)) return fail(ctx, POE_EIO, name);
            std::snprintf(name, sizeof name, "vx%05i.vxo", (int)done);
            if ((st = poe_get_field(ctx, shot, POE_F_VX, snap.data())) != POE_OK) return fail(ctx, st, "vx");
            if (!write_raw(path(o.out_dir, name), snap.data(), n)) return fail(ctx, POE_EIO, name);
        }
        std::printf("\nStep = %5d\n", (int)done);
    }
    // NSTEP rows; rows past the steps run stay 0, as the reference's cleared arrays do
    std::vector<float> tr((size_t)nstep * nrec, 0.0f);
    if ((st = poe_get_traces(ctx, shot, tr.data(), (int64_t)tr.size())) != POE_OK) return fail(ctx, st, "traces");
    poe_destroy(ctx);

    // trace columns: VSP vz, VSP vx, horizontal vz, horizontal vx, then the
    // vz points y = 50, a0_pos (.ats), a1_pos (.bwh), JSOURCE (.src)
    const int F = (int)f0;
    const int c_vsp = 0, c_hor = 2 * o.panj, c_pts = 2 * o.panj + 2 * o.panj2;
    bool ok = true;
    std::snprintf(name, sizeof name, "recvspvz%08i.vsp", F);
    ok = ok && write_rows(path(o.out_dir, name), tr, nstep, nrec, c_vsp, o.panj);
    std::snprintf(name, sizeof name, "recvspvx%08i.vsp", F);
    ok = ok && write_rows(path(o.out_dir, name), tr, nstep, nrec, c_vsp + o.panj, o.panj);
    std::snprintf(name, sizeof name, "rechorvz%08i.hor", F);
    ok = ok && write_rows(path(o.out_dir, name), tr, nstep, nrec, c_hor, o.panj2);
    std::snprintf(name, sizeof name, "rechorvx%08i.hor", F);
    ok = ok && write_rows(path(o.out_dir, name), tr, nstep, nrec, c_hor + o.panj2, o.panj2);
    const char *ext[3][2] = {{"recats", "ats"}, {"recbwh", "bwh"}, {"recsrc", "src"}};
    for (int i = 0; i < 3; ++i) {
        if (f0 < 1.0f) std::snprintf(name, sizeof name, "%s%08f.%s", ext[i][0], f0, ext[i][1]);
        else std::snprintf(name, sizeof name, "%s%08i.%s", ext[i][0], F, ext[i][1]);
        ok = ok && write_line(path(o.out_dir, name), tr, nstep, nrec, c_pts + 1 + i);
    }
    if (!ok) {
        std::cerr << "writing the receiver files failed\n";
        return 1;
    }
    return 0;
}
