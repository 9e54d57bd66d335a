// Host-side input/output of the drop-in interface, written portably in place of the
// reference's MFC / Win32 code: the parameter file (K:8541-8571), the direction file
// (K:8615-8649), the Tecplot acceleration reader (K:8708-8792), the Bernoulli initial face
// (K:8805-8811) and the pressure / curl writers (K:8916-8958).  Also an icosphere
// generator that reproduces the direction sets the reference ships.
//
// The Tecplot files hold one text row per voxel (about 160 bytes at 10 columns: 2.7 GB at
// 256^3), so the reader and the writers are parallel: the reader takes the file in 256 MB
// blocks, cuts each block's complete lines into one chunk per thread, counts the chunks'
// lines, then parses every chunk in place (strtod on the row text, rounded to float, as
// the reference's _wtof into float arrays); the writers format blocks of rows in parallel
// and write them in order.  OMNI3D_IO_THREADS sets the thread count (default: all
// hardware threads), OMNI3D_IO_BLOCK the reader's block size in bytes (default 256 MB).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
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

// Threads of the text readers and writers.
int io_threads()
{
    const char *e = std::getenv("OMNI3D_IO_THREADS");
    int n = e ? std::atoi(e) : (int)std::thread::hardware_concurrency();
    return std::max(1, std::min(n, 256));
}

// f(t) for t in [0, n): t = 0 on the calling thread.
template <typename F>
void parallel_for(int n, F &&f)
{
    if (n <= 1) {
        f(0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve((size_t)n - 1);
    for (int t = 1; t < n; t++) th.emplace_back([&f, t]() { f(t); });
    f(0);
    for (auto &x : th) x.join();
}

inline bool is_sep(char c) { return c == ' ' || c == '\t' || c == ','; }

// Where a Tecplot reader puts each voxel's columns, and what it found.
struct TecplotJob {
    const omni3d_file_params *fp;
    float *out[10];          // x y z u v w ax ay az mask (any may be NULL)
    long long rows_org;      // rows of the uncropped grid
};

struct ChunkResult {
    int ncol = -1;            // columns of the chunk's first row inside the crop
    long long bad_row = -1;   // first row inside the crop whose column count differs
};

// Parse the complete lines in [b, e) -- the chunk's first line is body row row0 -- into the
// job's arrays.  Rows outside the crop are skipped without being read, as in the reference.
ChunkResult parse_rows(const char *b, const char *e, long long row0, const TecplotJob &J)
{
    ChunkResult R;
    const omni3d_file_params *fp = J.fp;
    const long long nxo = fp->nx_org, nyo = fp->ny_org;
    const int i0 = fp->roi[0], i1 = fp->roi[1], j0 = fp->roi[2], j1 = fp->roi[3], k0 = fp->roi[4], k1 = fp->roi[5];
    const long long nx = i1 - i0 + 1, ny = j1 - j0 + 1;
    long long row = row0;
    for (const char *p = b; p < e && row < J.rows_org; row++) {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(e - p)));
        const char *le = nl ? nl : e;
        const char *next = nl ? nl + 1 : e;
        const long long i = row % nxo, j = (row / nxo) % nyo, k = row / (nxo * nyo);
        if (i >= i0 && i <= i1 && j >= j0 && j <= j1 && k >= k0 && k <= k1) {
            const char *te = le;
            while (te > p && te[-1] == '\r') te--;  // the line's end, as read_line strips it
            const char *tok[11];
            int n = 0;
            for (const char *q = p; q < te;) {
                while (q < te && is_sep(*q)) q++;
                if (q >= te) break;
                if (n < 11) tok[n] = q;
                n++;
                while (q < te && !is_sep(*q)) q++;
            }
            if (R.ncol < 0) R.ncol = n;
            if (n != R.ncol || (n != 10 && n != 7)) {
                R.bad_row = row;
                return R;
            }
            const long long ind = (i - i0) + (j - j0) * nx + (k - k0) * nx * ny;
            // strtod stops at the separator or line end that follows each token
            auto val = [&](int c) { return (float)std::strtod(tok[c], nullptr); };
            float **o = const_cast<float **>(J.out);
            if (o[0]) o[0][ind] = val(0);
            if (o[1]) o[1][ind] = val(1);
            if (o[2]) o[2][ind] = val(2);
            const int a = n == 10 ? 6 : 3;
            for (int c = 0; c < 3; c++)
                if (o[3 + c]) o[3 + c][ind] = n == 10 ? val(3 + c) : 0.0f;
            for (int c = 0; c < 4; c++)
                if (o[6 + c]) o[6 + c][ind] = val(a + c);
        }
        p = next;
    }
    return R;
}

// Rows [r0, r1) of `cols` columns printed "%15.9f" and separated by blanks, one per line.
void format_rows(std::string &buf, const float *const *cols, int ncols, long long r0, long long r1)
{
    buf.clear();
    buf.reserve((size_t)(r1 - r0) * (size_t)(16 * ncols + 1));
    char tmp[96];
    for (long long r = r0; r < r1; r++)
        for (int c = 0; c < ncols; c++) {
            int len = std::snprintf(tmp, sizeof(tmp), c + 1 < ncols ? "%15.9f " : "%15.9f\n", (double)cols[c][r]);
            if (len < (int)sizeof(tmp)) {
                buf.append(tmp, (size_t)len);
            } else {  // very large values print more than the buffer holds
                std::vector<char> big((size_t)len + 1);
                std::snprintf(big.data(), big.size(), c + 1 < ncols ? "%15.9f " : "%15.9f\n", (double)cols[c][r]);
                buf.append(big.data(), (size_t)len);
            }
        }
}

// The body of a Tecplot writer: V rows, formatted in parallel blocks, written in order.
bool write_rows(FILE *f, const float *const *cols, int ncols, long long V)
{
    const int T = io_threads();
    const long long block = 1LL << 20;
    std::vector<std::string> bufs((size_t)T);
    for (long long b0 = 0; b0 < V; b0 += block) {
        const long long b1 = std::min(V, b0 + block);
        const long long per = (b1 - b0 + T - 1) / T;
        parallel_for(T, [&](int t) {
            const long long r0 = std::min(b1, b0 + per * t), r1 = std::min(b1, r0 + per);
            format_rows(bufs[(size_t)t], cols, ncols, r0, r1);
        });
        for (int t = 0; t < T; t++)
            if (!bufs[(size_t)t].empty() && std::fwrite(bufs[(size_t)t].data(), 1, bufs[(size_t)t].size(), f) != bufs[(size_t)t].size())
                return false;
    }
    return true;
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
    TecplotJob J;
    J.fp = fp;
    float *outs[10] = {x, y, z, u, v, w, ax, ay, az, mask};
    std::copy(outs, outs + 10, J.out);
    J.rows_org = (long long)fp->nx_org * fp->ny_org * fp->nz_org;
    const int T = io_threads();
    const char *eb = std::getenv("OMNI3D_IO_BLOCK");
    size_t kBlock = eb ? std::max<size_t>(16, (size_t)std::strtoull(eb, nullptr, 10)) : ((size_t)256 << 20);
    if (std::fseek(f, 0, SEEK_END) == 0) {  // no larger than the file
        const long sz = std::ftell(f);
        if (sz >= 0) kBlock = std::min(kBlock, (size_t)sz + 1);
        std::fseek(f, 0, SEEK_SET);
    }
    // an uninitialised buffer (a zero-filled one would cost a pass over every block)
    size_t cap = kBlock;
    std::unique_ptr<char[]> buf(new char[cap]);
    size_t have = 0;            // bytes of buf holding unprocessed text
    int header = 0;             // header lines consumed
    long long rows = 0;         // body rows consumed
    int ncol = -1;
    long long bad_row = -1;
    bool eof = false;
    std::vector<ChunkResult> res((size_t)T);
    std::vector<long long> first((size_t)T + 1);
    std::vector<size_t> cut((size_t)T + 1);
    while (rows < J.rows_org && bad_row < 0) {
        if (!eof) {
            if (have + kBlock > cap) {  // a line longer than a block: grow
                std::unique_ptr<char[]> bigger(new char[have + kBlock]);
                std::memcpy(bigger.get(), buf.get(), have);
                buf.swap(bigger);
                cap = have + kBlock;
            }
            const size_t got = std::fread(buf.get() + have, 1, kBlock, f);
            have += got;
            if (got < kBlock) eof = true;
        }
        const char *base = buf.get();
        // complete lines end at the last newline; at end of file the rest is a line too
        size_t end = have;
        if (!eof) {
            const char *lastnl = nullptr;
            for (size_t q = have; q > 0; q--)
                if (base[q - 1] == '\n') { lastnl = base + q - 1; break; }
            if (!lastnl) {
                if (have > ((size_t)1 << 31)) { std::fclose(f); return io_fail(OMNI3D_ERR_IO, std::string(path) + ": line too long"); }
                continue;  // read more
            }
            end = (size_t)(lastnl - base) + 1;
        }
        size_t pos = 0;
        while (header < 3 && pos < end) {  // the three header lines
            const char *nl = static_cast<const char *>(std::memchr(base + pos, '\n', end - pos));
            pos = nl ? (size_t)(nl - base) + 1 : end;
            header++;
        }
        if (header < 3) {
            if (eof) { std::fclose(f); return io_fail(OMNI3D_ERR_IO, std::string(path) + ": short header"); }
        } else if (pos < end) {
            // one chunk per thread, cut after a newline; count lines, then parse in parallel
            cut[0] = pos;
            for (int t = 1; t < T; t++) {
                size_t c = pos + (end - pos) * (size_t)t / (size_t)T;
                c = std::max(c, cut[(size_t)t - 1]);
                const char *nl = c < end ? static_cast<const char *>(std::memchr(base + c, '\n', end - c)) : nullptr;
                cut[(size_t)t] = nl ? (size_t)(nl - base) + 1 : end;
            }
            cut[(size_t)T] = end;
            std::vector<long long> nlines((size_t)T, 0);
            parallel_for(T, [&](int t) {
                long long n = 0;
                const char *p = base + cut[(size_t)t], *e = base + cut[(size_t)t + 1];
                while (p < e) {
                    const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(e - p)));
                    n++;
                    p = nl ? nl + 1 : e;
                }
                nlines[(size_t)t] = n;
            });
            first[0] = rows;
            for (int t = 0; t < T; t++) first[(size_t)t + 1] = first[(size_t)t] + nlines[(size_t)t];
            parallel_for(T, [&](int t) {
                res[(size_t)t] = parse_rows(base + cut[(size_t)t], base + cut[(size_t)t + 1], first[(size_t)t], J);
            });
            for (int t = 0; t < T && bad_row < 0; t++) {  // the first inconsistency in row order
                const ChunkResult &r = res[(size_t)t];
                if (r.ncol < 0) continue;
                if (ncol < 0) ncol = r.ncol;
                if (r.ncol != ncol) bad_row = first[(size_t)t];
                else if (r.bad_row >= 0) bad_row = r.bad_row;
            }
            rows = first[(size_t)T];
        }
        // keep the incomplete last line for the next block
        std::memmove(buf.get(), buf.get() + end, have - end);
        have -= end;
        if (eof && have == 0) break;
    }
    std::fclose(f);
    if (bad_row >= 0 || (ncol >= 0 && ncol != 10 && ncol != 7))
        return io_fail(OMNI3D_ERR_IO, std::string(path) + ": rows must have 10 (x y z u v w Du Dv Dw mask) "
                                                          "or 7 (x y z Du Dv Dw mask) columns");
    if (rows < J.rows_org) return io_fail(OMNI3D_ERR_IO, std::string(path) + ": fewer rows than the grid");
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
    const float *cols[5] = {x, y, z, p, count};
    bool ok = write_rows(f, cols, 5, V);  // rows "%15.9f %15.9f %15.9f %15.9f %15.9f\n" (K:8929)
    int bad = !ok || std::ferror(f);
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
    const float *cols[4] = {x, y, z, curl};
    bool ok = write_rows(f, cols, 4, V);  // rows "%15.9f %15.9f %15.9f %15.9f\n" (K:8954)
    int bad = !ok || std::ferror(f);
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
