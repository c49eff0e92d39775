// cnv_io.cpp -- the reference's run outputs from device results: log lines and VTK files.
//
// Log lines (src/poisson.c:212/:275 and src/main.c:401-414): every time step of the
// reference writes one line from its Poisson solver and two progress lines. The per-step
// record cnv_step fills (iteration count, stop norm, continuity max/min) carries every value
// these lines print except the timings, which the caller measures; so a GPU run writes a log
// that diffs against the reference's line by line (timings aside).
//
// VTK files (src/utils.c:38-99): ASCII STRUCTURED_POINTS, "%.6lf" per value, rows of the field
// on separate lines, file name "<dir>/<title>-1-<count>.vtk" with one counter shared by every
// field the run writes, opened for append as the reference does.
#include <sys/stat.h>
#include <sys/types.h>

#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cnv_internal.h"

using namespace cnv;

namespace {

int ifail(int status, const std::string& m) {
    set_last_error(m.c_str());
    return status;
}

int put(char* buf, size_t len, const std::string& s) {
    if (!buf || len == 0) return ifail(CNV_BAD_ARG, "null or empty output buffer");
    if (s.size() + 1 > len) return ifail(CNV_BAD_ARG, "output buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return CNV_OK;
}

std::string fmt(const char* f, ...) __attribute__((format(printf, 1, 2)));
std::string fmt(const char* f, ...) {
    char tmp[512];
    va_list ap;
    va_start(ap, f);
    vsnprintf(tmp, sizeof tmp, f, ap);
    va_end(ap);
    return tmp;
}

// mkdir -p
int make_dirs(const std::string& path) {
    std::string cur;
    for (size_t i = 0; i <= path.size(); ++i) {
        if (i == path.size() || path[i] == '/') {
            if (!cur.empty() && cur != "." && cur != "..") {
                if (mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) return -1;
            }
        }
        if (i < path.size()) cur += path[i];
    }
    return 0;
}

}  // namespace

extern "C" {

int cnv_format_step_log(const cnv_step_info* info, int t, double dt, int it_max, double iter_seconds,
                        double elapsed_seconds, char* buf, size_t len) {
    if (!info) return ifail(CNV_BAD_ARG, "null step record");
    std::string s;
    if (info->status == CNV_NOT_CONVERGED)
        s = "Error: maximum number of iterations achieved for Poisson equation.\n";
    else
        s = fmt("Poisson equation solved with %d iterations - root-sum-of-squares error: %E\n", info->iters,
                info->err);
    if (info->status == CNV_OK) {
        s += fmt("Iteration: %d | ", t);
        s += fmt("Time: %lf | ", (double)t * dt);
        s += fmt("Progress: %.2lf%% | ", (double)100 * t / it_max);
        s += fmt("Iter time: %.3f s\n", iter_seconds);
        s += fmt("Continuity max: %E | ", info->cont_max);
        s += fmt("Continuity min: %E | ", info->cont_min);
        s += fmt("Elapsed: %.1f s | ", elapsed_seconds);
        if (t > 0)
            s += fmt("Est. remaining: %.1f s\n", elapsed_seconds / (t + 1) * (it_max - t));
        else
            s += "Est. remaining: -- s\n";
    }
    return put(buf, len, s);
}

int cnv_write_vtk(const char* output_dir, const char* title, int count, const double* field, int m, int n) {
    if (!output_dir || !title || !field || m < 1 || n < 1) return ifail(CNV_BAD_ARG, "bad VTK arguments");
    if (make_dirs(output_dir) != 0) return ifail(CNV_IO_ERROR, std::string("cannot create ") + output_dir);
    const std::string name = fmt("%s/%s-1-%d.vtk", output_dir, title, count);
    FILE* pf = std::fopen(name.c_str(), "a");
    if (!pf) return ifail(CNV_IO_ERROR, "Error while opening file: " + name);
    std::fprintf(pf, "# vtk DataFile Version 2.0\n");
    std::fprintf(pf, "test\n");
    std::fprintf(pf, "ASCII\n");
    std::fprintf(pf, "DATASET STRUCTURED_POINTS\n");
    std::fprintf(pf, "DIMENSIONS %d %d 1\n", m, n);
    std::fprintf(pf, "ORIGIN 0 0 0\n");
    std::fprintf(pf, "SPACING 1 1 1\n");
    std::fprintf(pf, "POINT_DATA %d\n", m * n);
    std::fprintf(pf, "SCALARS values float\n");
    std::fprintf(pf, "LOOKUP_TABLE default");
    std::vector<char> line;
    char c[352];  // "%.6lf" of the largest double needs 317 characters plus the separator
    for (int i = 0; i < m; ++i) {
        line.clear();
        line.push_back('\n');
        for (int j = 0; j < n; ++j) {
            int k = std::snprintf(c, sizeof c, j == 0 ? "%.6lf" : " %.6lf", field[(size_t)i * n + j]);
            if (k < 0) k = 0;
            if (k > (int)sizeof c - 1) k = (int)sizeof c - 1;
            line.insert(line.end(), c, c + k);
        }
        std::fwrite(line.data(), 1, line.size(), pf);
    }
    const bool bad = std::ferror(pf) != 0;
    if (std::fclose(pf) != 0 || bad) return ifail(CNV_IO_ERROR, "write failed: " + name);
    return CNV_OK;
}

}  // extern "C"
