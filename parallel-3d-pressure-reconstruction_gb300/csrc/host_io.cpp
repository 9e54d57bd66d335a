// Host-side input/output of the drop-in interface, written portably in place of the
// reference's MFC / Win32 code: the parameter file (K:8541-8571), the direction file
// (K:8615-8649), the Tecplot acceleration reader (K:8708-8792), the Bernoulli initial face
// (K:8805-8811) and the pressure / curl writers (K:8916-8958).  Also an icosphere
// generator that reproduces the direction sets the reference ships.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "omni3d.h"

namespace omni3d {
void set_global_error(const std::string &msg);  // api.cu
}

namespace {

int io_fail(int code, const std::string &msg)
{
    omni3d::set_global_error(msg);
    return code;
}

// One line without its end-of-line characters; false at end of file.
bool read_line(FILE *f, std::string &s)
{
    s.clear();
    int c;
    bool any = false;
    while ((c = std::fgetc(f)) != EOF) {
        any = true;
        if (c == '\n') break;
        s.push_back((char)c);
    }
    while (!s.empty() && (s.back() == '\r' || s.back() == '\n')) s.pop_back();
    return any;
}

// _wtoi / _wtof semantics: leading blanks, then the longest numeric prefix, else 0.
int to_int(const std::string &s) { return std::atoi(s.c_str()); }
double to_double(const std::string &s) { return std::strtod(s.c_str(), nullptr); }

void copy_str(char *dst, size_t cap, const std::string &s)
{
    size_t n = std::min(cap - 1, s.size());
    std::memcpy(dst, s.data(), n);
    dst[n] = 0;
}

std::vector<std::string> tokens(const std::string &s)
{
    std::vector<std::string> t;
    size_t i = 0, n = s.size();
    while (i < n) {
        while (i < n && (s[i] == ' ' || s[i] == '\t' || s[i] == ',')) i++;
        size_t j = i;
        while (j < n && !(s[j] == ' ' || s[j] == '\t' || s[j] == ',')) j++;
        if (j > i) t.push_back(s.substr(i, j - i));
        i = j;
    }
    return t;
}

}  // namespace

extern "C" {

int omni3d_read_params(const char *path, omni3d_file_params *out)
{
    if (!path || !out) return io_fail(OMNI3D_ERR_ARG, "NULL argument");
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(OMNI3D_ERR_IO, std::string("Parameter input file: \"") + path + "\" open error");
    std::memset(out, 0, sizeof(*out));
    std::string s;
    auto next = [&](std::string &dst) { if (!read_line(f, dst)) dst.clear(); };
    std::string L[22];
    for (auto &l : L) next(l);
    std::fclose(f);
    out->nx_org = to_int(L[0]);
    out->ny_org = to_int(L[1]);
    out->nz_org = to_int(L[2]);
    out->dx = (float)to_double(L[3]);
    out->dy = (float)to_double(L[4]);
    out->dz = (float)to_double(L[5]);
    out->density = (float)to_double(L[6]);
    out->scale = (float)to_int(L[7]);
    out->line_spacing = (float)to_double(L[8]);
    out->n_dirs = to_int(L[9]);
    copy_str(out->dir_file, sizeof(out->dir_file), L[10]);
    copy_str(out->accel_dir, sizeof(out->accel_dir), L[11]);
    copy_str(out->pressure_dir, sizeof(out->pressure_dir), L[12]);
    out->n_iter = to_int(L[13]);
    out->threshold = (float)to_double(L[14]);
    // hidden lines (K:8564-8570): blank -> default
    out->pref = L[15].empty() ? 0.0f : (float)to_double(L[15]);
    out->roi[0] = L[16].empty() ? 0 : to_int(L[16]);
    out->roi[1] = L[17].empty() ? out->nx_org - 1 : to_int(L[17]);
    out->roi[2] = L[18].empty() ? 0 : to_int(L[18]);
    out->roi[3] = L[19].empty() ? out->ny_org - 1 : to_int(L[19]);
    out->roi[4] = L[20].empty() ? 0 : to_int(L[20]);
    out->roi[5] = L[21].empty() ? out->nz_org - 1 : to_int(L[21]);
    if (out->nx_org < 1 || out->ny_org < 1 || out->nz_org < 1)
        return io_fail(OMNI3D_ERR_IO, "parameter file: grid size must be positive");
    for (int a = 0; a < 3; a++) {
        int lo = out->roi[2 * a], hi = out->roi[2 * a + 1];
        int n = a == 0 ? out->nx_org : (a == 1 ? out->ny_org : out->nz_org);
        if (lo < 0 || hi >= n || hi < lo) return io_fail(OMNI3D_ERR_IO, "parameter file: region of interest out of range");
    }
    return OMNI3D_OK;
}

int omni3d_read_directions(const char *path, int n, float *out)
{
    if (!path || !out || n <= 0) return io_fail(OMNI3D_ERR_ARG, "bad arguments");
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(OMNI3D_ERR_IO, std::string("Virtual grid points:") + path + " open error");
    std::string s;
    int got = 0;
    while (got < n && read_line(f, s)) {
        std::vector<std::string> t = tokens(s);
        if (t.size() < 3) break;  // the trailing count row, or a short file
        // the reference takes the last three fields of the row (K:8626-8647)
        size_t m = t.size();
        out[3 * got + 0] = (float)to_double(t[m - 3]);
        out[3 * got + 1] = (float)to_double(t[m - 2]);
        out[3 * got + 2] = (float)to_double(t[m - 1]);
        got++;
    }
    std::fclose(f);
    if (got < n) return io_fail(OMNI3D_ERR_IO, std::string("direction file ") + path + ": fewer rows than requested");
    return got;
}

int omni3d_read_tecplot(const char *path, const omni3d_file_params *fp, float *x, float *y, float *z, float *u,
                        float *v, float *w, float *ax, float *ay, float *az, float *mask)
{
    if (!path || !fp) return io_fail(OMNI3D_ERR_ARG, "bad arguments");
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(OMNI3D_ERR_IO, std::string(path) + " failed to open");
    std::string s;
    for (int h = 0; h < 3; h++)
        if (!read_line(f, s)) { std::fclose(f); return io_fail(OMNI3D_ERR_IO, std::string(path) + ": short header"); }
    const int i0 = fp->roi[0], i1 = fp->roi[1], j0 = fp->roi[2], j1 = fp->roi[3], k0 = fp->roi[4], k1 = fp->roi[5];
    const long long nx = i1 - i0 + 1, ny = j1 - j0 + 1;
    int ncol = -1;
    for (long long k = 0; k < fp->nz_org; k++)
        for (long long j = 0; j < fp->ny_org; j++)
            for (long long i = 0; i < fp->nx_org; i++) {
                if (!read_line(f, s)) {
                    std::fclose(f);
                    return io_fail(OMNI3D_ERR_IO, std::string(path) + ": fewer rows than the grid");
                }
                if (!(i >= i0 && i <= i1 && j >= j0 && j <= j1 && k >= k0 && k <= k1)) continue;
                std::vector<std::string> t = tokens(s);
                if (ncol < 0) ncol = (int)t.size();
                if ((int)t.size() != ncol || (ncol != 10 && ncol != 7)) {
                    std::fclose(f);
                    return io_fail(OMNI3D_ERR_IO, std::string(path) + ": rows must have 10 (x y z u v w Du Dv Dw mask) "
                                                                      "or 7 (x y z Du Dv Dw mask) columns");
                }
                long long ind = (i - i0) + (j - j0) * nx + (k - k0) * nx * ny;
                auto val = [&](int c) { return (float)to_double(t[c]); };
                if (x) x[ind] = val(0);
                if (y) y[ind] = val(1);
                if (z) z[ind] = val(2);
                int o = ncol == 10 ? 6 : 3;
                if (ncol == 10) {
                    if (u) u[ind] = val(3);
                    if (v) v[ind] = val(4);
                    if (w) w[ind] = val(5);
                } else {
                    if (u) u[ind] = 0.0f;
                    if (v) v[ind] = 0.0f;
                    if (w) w[ind] = 0.0f;
                }
                if (ax) ax[ind] = val(o);
                if (ay) ay[ind] = val(o + 1);
                if (az) az[ind] = val(o + 2);
                if (mask) mask[ind] = val(o + 3);
            }
    std::fclose(f);
    return ncol;
}

int omni3d_bernoulli_face(int nx, int ny, int nz, float pref, float density, const float *u, const float *v,
                          const float *w, float *p_init)
{
    if (!u || !v || !w || !p_init || nx < 1 || ny < 1 || nz < 1) return io_fail(OMNI3D_ERR_ARG, "bad arguments");
    long long V = (long long)nx * ny * nz;
    std::fill(p_init, p_init + V, 0.0f);
    for (long long i = 0; i < nx; i++)
        for (long long k = 0; k < nz; k++) {
            long long ind = i + k * (long long)nx * ny;
            p_init[ind] = (float)(pref - 0.5 * density * (u[ind] * u[ind] + v[ind] * v[ind] + w[ind] * w[ind]));
        }
    return OMNI3D_OK;
}

int omni3d_write_pressure(const char *path, int nx, int ny, int nz, const float *x, const float *y, const float *z,
                          const float *p, const float *count)
{
    if (!path || !x || !y || !z || !p || !count) return io_fail(OMNI3D_ERR_ARG, "NULL argument");
    FILE *f = std::fopen(path, "wb");
    if (!f) return io_fail(OMNI3D_ERR_IO, std::string(path) + ": cannot create");
    std::fprintf(f, "TITLE = \"Pressure Integrated From GPU Based Omni 3D Method\"\n");
    std::fprintf(f, "VARIABLES = \"X\",\"Y\",\"Z\",\"P\",\"Count\"\n");
    std::fprintf(f, "ZONE I=%i, J=%i, K=%i,F=POINT\n", nx, ny, nz);
    long long V = (long long)nx * ny * nz;
    for (long long i = 0; i < V; i++)
        std::fprintf(f, "%15.9f %15.9f %15.9f %15.9f %15.9f\n", x[i], y[i], z[i], p[i], count[i]);
    int bad = std::ferror(f);
    std::fclose(f);
    return bad ? io_fail(OMNI3D_ERR_IO, std::string(path) + ": write error") : OMNI3D_OK;
}

int omni3d_write_curl(const char *path, int nx, int ny, int nz, const float *x, const float *y, const float *z,
                      const float *curl)
{
    if (!path || !x || !y || !z || !curl) return io_fail(OMNI3D_ERR_ARG, "NULL argument");
    FILE *f = std::fopen(path, "wb");
    if (!f) return io_fail(OMNI3D_ERR_IO, std::string(path) + ": cannot create");
    std::fprintf(f, "TITLE = \"Curl of Material Acceleration Multiplied by the Mask\"\n");
    std::fprintf(f, "VARIABLES = \"X\",\"Y\",\"Z\",\"Curl of Acceleration\"\n");
    std::fprintf(f, "ZONE I=%i, J=%i, K=%i,F=POINT\n", nx, ny, nz);
    long long V = (long long)nx * ny * nz;
    for (long long i = 0; i < V; i++) std::fprintf(f, "%15.9f %15.9f %15.9f %15.9f\n", x[i], y[i], z[i], curl[i]);
    int bad = std::ferror(f);
    std::fclose(f);
    return bad ? io_fail(OMNI3D_ERR_IO, std::string(path) + ": write error") : OMNI3D_OK;
}

// Icosphere: an icosahedron with poles on z, the lower ring at z = -1/sqrt(5) and the upper
// ring, rotated by 36 degrees, at z = 0.46000602 -- the base the reference's
// GridIcosahedronDivide*.dat files are subdivided from (their 42-, 162- and 642-vertex
// sets are reproduced exactly) -- refined by recursive edge-midpoint subdivision with
// projection onto the unit sphere, printed with six decimals and sorted by (x, y, z).
int omni3d_icosphere(int level, float *out, int cap)
{
    if (level < 1 || level > 9) return io_fail(OMNI3D_ERR_RANGE, "icosphere level must be 1..9");
    const double PI = 3.14159265358979323846;
    const double zl = -1.0 / std::sqrt(5.0), rl = 2.0 / std::sqrt(5.0);
    const double zu = 0.46000602, ru = std::sqrt(1.0 - zu * zu);
    std::vector<std::array<double, 3>> V;
    V.push_back({0.0, 0.0, 1.0});
    V.push_back({0.0, 0.0, -1.0});
    for (int k = 0; k < 5; k++) V.push_back({rl * std::cos(2 * PI * k / 5), rl * std::sin(2 * PI * k / 5), zl});
    for (int k = 0; k < 5; k++)
        V.push_back({ru * std::cos(2 * PI * k / 5 + PI / 5), ru * std::sin(2 * PI * k / 5 + PI / 5), zu});
    std::vector<std::array<int, 3>> F;
    for (int k = 0; k < 5; k++) {
        int a = 2 + k, b = 2 + (k + 1) % 5, ua = 7 + k, ub = 7 + (k + 1) % 5;
        F.push_back({1, b, a});
        F.push_back({0, ua, ub});
        F.push_back({a, b, ua});
        F.push_back({b, ub, ua});
    }
    for (int l = 1; l < level; l++) {
        std::map<std::pair<int, int>, int> mid;
        auto midpoint = [&](int a, int b) {
            std::pair<int, int> key(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            std::array<double, 3> m = {V[a][0] + V[b][0], V[a][1] + V[b][1], V[a][2] + V[b][2]};
            double n = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            V.push_back({m[0] / n, m[1] / n, m[2] / n});
            mid[key] = (int)V.size() - 1;
            return (int)V.size() - 1;
        };
        std::vector<std::array<int, 3>> G;
        G.reserve(F.size() * 4);
        for (auto &t : F) {
            int ab = midpoint(t[0], t[1]), bc = midpoint(t[1], t[2]), ca = midpoint(t[2], t[0]);
            G.push_back({t[0], ab, ca});
            G.push_back({t[1], bc, ab});
            G.push_back({t[2], ca, bc});
            G.push_back({ab, bc, ca});
        }
        F.swap(G);
    }
    // six-decimal text, as in the files, read back the way the reference reads it
    std::vector<std::array<double, 3>> R(V.size());
    char buf[128];
    for (size_t i = 0; i < V.size(); i++) {
        std::snprintf(buf, sizeof(buf), "%f %f %f", V[i][0], V[i][1], V[i][2]);
        char *e1, *e2;
        R[i][0] = std::strtod(buf, &e1);
        R[i][1] = std::strtod(e1, &e2);
        R[i][2] = std::strtod(e2, nullptr);
    }
    std::stable_sort(R.begin(), R.end());
    int n = (int)R.size();
    if (out) {
        for (int i = 0; i < std::min(n, cap); i++)
            for (int a = 0; a < 3; a++) out[3 * i + a] = (float)R[i][a];
    }
    return n;
}

}  // extern "C"
