// omni3d: drop-in replacement of the reference executable (K:8467-8984).
//
// Reads Parameter_Omni3D.dat from the working directory (or --params PATH), the direction
// file it names, and every acceleration file in its acceleration folder (sorted by path,
// recursively, as `dir /B /S` lists them); writes <pressure folder>/PressureOmni3D_%05d.dat
// per input, CurlofMaterialAcc_Sample.dat for the first input, and log.dat.  Windows path
// separators in the parameter file are accepted.  Defaults follow the reference main(): the
// selected method, exactly NoItr iterations, no gauge.
//
// Options: --params PATH  --method select|plain|weighted|weighted-fixed-bc|select-fixed-bc|
//                                   mini-curl|weighted-mini-curl
//          --solver anchor|sweep  --tol T
//          --gauge none|point|mean  --ref I,J,K  --grad f32|bf16  --device N
//          --autotune (time a few line orders for this grid before the first snapshot)
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "omni3d.h"

namespace {

std::string fix_path(std::string s)
{
    for (char &c : s)
        if (c == '\\') c = '/';
    while (!s.empty() && (s.back() == ' ' || s.back() == '\t')) s.pop_back();
    return s;
}

bool is_dir(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

void list_files(const std::string &dir, std::vector<std::string> &out)
{
    DIR *d = opendir(dir.c_str());
    if (!d) return;
    std::vector<std::string> names;
    while (struct dirent *e = readdir(d)) {
        std::string n = e->d_name;
        if (n == "." || n == "..") continue;
        names.push_back(n);
    }
    closedir(d);
    std::sort(names.begin(), names.end());
    for (const std::string &n : names) {
        std::string p = dir + (dir.empty() || dir.back() == '/' ? "" : "/") + n;
        if (is_dir(p)) list_files(p, out);
        else out.push_back(p);
    }
}

int usage()
{
    std::fprintf(stderr,
                 "usage: omni3d [--params PATH] [--method select|plain|weighted|weighted-fixed-bc|select-fixed-bc|\n"
                 "              mini-curl|weighted-mini-curl] [--solver anchor|sweep] [--tol T]\n"
                 "              [--gauge none|point|mean] [--ref I,J,K] [--grad f32|bf16] [--device N]\n"
                 "              [--autotune]\n");
    return 2;
}

}  // namespace

int main(int argc, char **argv)
{
    std::string params_path = "Parameter_Omni3D.dat";
    omni3d_params prm;
    omni3d_default_params(&prm);
    prm.method = OMNI3D_METHOD_SELECT;  // what the reference main() runs (K:8849)
    for (int a = 1; a < argc; a++) {
        std::string k = argv[a];
        auto val = [&]() -> std::string {
            if (a + 1 >= argc) { usage(); std::exit(2); }
            return argv[++a];
        };
        if (k == "--params") params_path = val();
        else if (k == "--method") {
            std::string v = val();
            if (v == "plain") prm.method = OMNI3D_METHOD_PLAIN;
            else if (v == "select") prm.method = OMNI3D_METHOD_SELECT;
            else if (v == "weighted") prm.method = OMNI3D_METHOD_WEIGHTED;
            else if (v == "weighted-fixed-bc") prm.method = OMNI3D_METHOD_WEIGHTED_FIXED_BC;
            else if (v == "select-fixed-bc") prm.method = OMNI3D_METHOD_SELECT_FIXED_BC;
            else if (v == "mini-curl") prm.method = OMNI3D_METHOD_MINI_CURL;
            else if (v == "weighted-mini-curl") prm.method = OMNI3D_METHOD_WEIGHTED_MINI_CURL;
            else return usage();
        }
        else if (k == "--solver") { std::string v = val(); prm.solver = v == "sweep" ? OMNI3D_SOLVER_SWEEP : OMNI3D_SOLVER_ANCHOR; }
        else if (k == "--tol") prm.tol = std::atof(val().c_str());
        else if (k == "--gauge") {
            std::string v = val();
            prm.gauge = v == "point" ? OMNI3D_GAUGE_POINT : (v == "mean" ? OMNI3D_GAUGE_MEAN : OMNI3D_GAUGE_NONE);
        } else if (k == "--ref") {
            std::string v = val();
            if (std::sscanf(v.c_str(), "%d,%d,%d", &prm.ref_i, &prm.ref_j, &prm.ref_k) != 3) return usage();
        } else if (k == "--grad") prm.grad_storage = val() == "bf16" ? OMNI3D_GRAD_BF16 : OMNI3D_GRAD_F32;
        else if (k == "--device") prm.device = std::atoi(val().c_str());
        else if (k == "--autotune") prm.autotune = 1;
        else return usage();
    }

    FILE *log = std::fopen("log.dat", "w");
    omni3d_file_params fp;
    if (omni3d_read_params(params_path.c_str(), &fp) != OMNI3D_OK) {
        std::printf("%s\n", omni3d_global_error());
        if (log) std::fclose(log);
        return 1;
    }
    const int nx = fp.roi[1] - fp.roi[0] + 1, ny = fp.roi[3] - fp.roi[2] + 1, nz = fp.roi[5] - fp.roi[4] + 1;
    const long long V = (long long)nx * ny * nz;

    std::printf("Reading virtual grid points on the sphere..........\n");
    std::vector<float> dirs(3 * (size_t)std::max(fp.n_dirs, 1));
    if (omni3d_read_directions(fix_path(fp.dir_file).c_str(), fp.n_dirs, dirs.data()) < 0) {
        std::printf("%s\n", omni3d_global_error());
        if (log) std::fclose(log);
        return 1;
    }
    std::printf("done\n");

    prm.nx = nx;
    prm.ny = ny;
    prm.nz = nz;
    prm.dx = fp.dx;
    prm.dy = fp.dy;
    prm.dz = fp.dz;
    prm.density = fp.density;
    prm.line_spacing = fp.line_spacing;
    prm.n_dirs = fp.n_dirs;
    prm.dirs = dirs.data();
    prm.max_iter = fp.n_iter;
    prm.threshold = fp.threshold;
    omni3d_ctx *ctx = nullptr;
    if (omni3d_create(&prm, &ctx) != OMNI3D_OK) {
        std::printf("%s\n", omni3d_global_error());
        if (log) std::fclose(log);
        return 1;
    }

    std::string acc_dir = fix_path(fp.accel_dir), out_dir = fix_path(fp.pressure_dir);
    if (!is_dir(acc_dir)) {
        std::printf("Acceleration folder does not exist: %s\n", fp.accel_dir);
        omni3d_destroy(ctx);
        if (log) std::fclose(log);
        return 1;
    }
    if (!is_dir(out_dir)) mkdir(out_dir.c_str(), 0755);
    std::vector<std::string> files;
    list_files(acc_dir, files);

    // Two slots of host buffers: while snapshot n is solved on the GPU, snapshot n + 1 is
    // parsed into the other slot and snapshot n - 1's output is written from it.
    struct Slot {
        std::vector<float> x, y, z, u, v, w, ax, ay, az, mask, p0, p, cnt;
        int ncol = -1;
        std::string err;
    };
    Slot slot[2];
    for (Slot &s : slot)
        for (auto *a : {&s.x, &s.y, &s.z, &s.u, &s.v, &s.w, &s.ax, &s.ay, &s.az, &s.mask, &s.p0, &s.p, &s.cnt})
            a->resize((size_t)V);
    std::vector<float> curl((size_t)V);
    auto read_into = [&](size_t fi, Slot &s) {
        s.ncol = omni3d_read_tecplot(files[fi].c_str(), &fp, s.x.data(), s.y.data(), s.z.data(), s.u.data(),
                                     s.v.data(), s.w.data(), s.ax.data(), s.ay.data(), s.az.data(), s.mask.data());
        s.err = s.ncol < 0 ? omni3d_global_error() : "";
    };
    std::printf("Processing Starts\n");
    if (log) std::fprintf(log, "Processing Starts\n");
    int rc_all = 0;
    std::thread reader, writer;
    if (!files.empty()) reader = std::thread(read_into, (size_t)0, std::ref(slot[0]));
    for (size_t fi = 0; fi < files.size(); fi++) {
        Slot &s = slot[fi % 2];
        reader.join();  // snapshot fi is parsed
        if (writer.joinable()) writer.join();  // the other slot is free again
        if (fi + 1 < files.size()) reader = std::thread(read_into, fi + 1, std::ref(slot[(fi + 1) % 2]));
        std::string name = files[fi].substr(files[fi].find_last_of('/') + 1);
        std::printf("%s\n", name.c_str());
        if (log) std::fprintf(log, "%s", name.c_str());
        if (s.ncol < 0) {
            if (log) std::fprintf(log, " failed to open\n");
            continue;
        }
        if (log) std::fprintf(log, "\n");
        omni3d_bernoulli_face(nx, ny, nz, fp.pref, fp.density, s.u.data(), s.v.data(), s.w.data(), s.p0.data());
        omni3d_stats stt;
        int rc = omni3d_solve(ctx, s.ax.data(), s.ay.data(), s.az.data(), nullptr, s.mask.data(), s.p0.data(),
                              s.p.data(), s.cnt.data(), 0, &stt);
        if (rc != OMNI3D_OK) {
            std::printf("CUDA error: %s\n", omni3d_last_error(ctx));
            rc_all = 1;
            continue;
        }
        if (fi == 0) {
            omni3d_curl(ctx, s.ax.data(), s.ay.data(), s.az.data(), s.mask.data(), curl.data(), 0);
            omni3d_write_curl("CurlofMaterialAcc_Sample.dat", nx, ny, nz, s.x.data(), s.y.data(), s.z.data(),
                              curl.data());
        }
        std::string out = out_dir + ((!out_dir.empty() && out_dir.back() != '/') ? "/" : "");
        char name_buf[64];
        std::snprintf(name_buf, sizeof(name_buf), "PressureOmni3D_%05d.dat", (int)fi);
        out += name_buf;
        writer = std::thread([&s, out, nx, ny, nz]() {
            if (omni3d_write_pressure(out.c_str(), nx, ny, nz, s.x.data(), s.y.data(), s.z.data(), s.p.data(),
                                      s.cnt.data()) != OMNI3D_OK)
                std::printf("%s\n", omni3d_global_error());
        });
        std::printf("  %d iterations, %lld lines, %.1f ms\n", stt.iterations, stt.n_lines, stt.ms_total);
    }
    if (reader.joinable()) reader.join();
    if (writer.joinable()) writer.join();
    omni3d_destroy(ctx);
    if (log) std::fclose(log);
    return rc_all;
}
