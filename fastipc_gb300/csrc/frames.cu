// Per-frame output of the driver: the Wavefront OBJ that write_image writes for 3D scenes
// (NEWTON_IPC.py:900-931).  Host code only.  The text is formatted in parallel chunks and written
// in order: the 177k-vertex bar takes about 50 ms on 8 cores against 0.33 s for the Python loop.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace {

// Python's '%.6f' (the reference's formatter) and C's agree on every finite double (both round
// the exact binary value correctly); they differ only for NaN, which C may print as "-nan".
inline void put_fixed6(std::string& out, double v) {
    char buf[64];
    if (isnan(v)) {
        out += "nan";
        return;
    }
    const int n = snprintf(buf, sizeof(buf), "%.6f", v);
    if (n > 0 && n < (int)sizeof(buf)) {
        out.append(buf, n);
    } else {   // |v| >= 1e56: the exact decimal expansion is longer than buf
        std::vector<char> big(n + 1);
        snprintf(big.data(), big.size(), "%.6f", v);
        out.append(big.data(), n);
    }
}

void format_vertices(const double* x, long long i0, long long i1, std::string& out) {
    out.reserve((size_t)(i1 - i0) * 40);
    for (long long i = i0; i < i1; ++i) {
        out += "v ";
        put_fixed6(out, x[3 * i]);
        out += ' ';
        put_fixed6(out, x[3 * i + 1]);
        out += ' ';
        put_fixed6(out, x[3 * i + 2]);
        out += '\n';
    }
}

void format_faces(const int* t, long long i0, long long i1, std::string& out) {
    out.reserve((size_t)(i1 - i0) * 24);
    char buf[48];
    for (long long i = i0; i < i1; ++i) {
        const int n = snprintf(buf, sizeof(buf), "f %d %d %d\n", t[3 * i] + 1, t[3 * i + 1] + 1, t[3 * i + 2] + 1);
        out.append(buf, n);
    }
}

}  // namespace

extern "C" {

// write_image for dim 3 (NEWTON_IPC.py:926-931): "v %.6f %.6f %.6f" per vertex, then
// "f %d %d %d" per boundary triangle with 1-based ids.  x_h [V][3], tris_h [F][3], host memory.
int fipc_write_obj(const char* path, int n_verts, const double* x_h, int n_tris, const int* tris_h) {
    if (!path || n_verts < 0 || n_tris < 0 || (n_verts > 0 && !x_h) || (n_tris > 0 && !tris_h)) return fipc::FIPC_ERR_ARGUMENT;
    const int hw = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const long long nv = n_verts, nf = n_tris;
    const int parts = (int)std::max(1LL, std::min<long long>(hw, (nv + nf) / 20000 + 1));
    std::vector<std::string> vtxt(parts), ftxt(parts);
    auto work = [&](int p) {
        format_vertices(x_h, nv * p / parts, nv * (p + 1) / parts, vtxt[p]);
        format_faces(tris_h, nf * p / parts, nf * (p + 1) / parts, ftxt[p]);
    };
    if (parts == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int p = 0; p < parts; ++p) th.emplace_back(work, p);
        for (auto& t : th) t.join();
    }
    FILE* f = fopen(path, "wb");
    if (!f) return fipc::FIPC_ERR_IO;
    bool ok = true;
    for (int p = 0; p < parts && ok; ++p) ok = fwrite(vtxt[p].data(), 1, vtxt[p].size(), f) == vtxt[p].size();
    for (int p = 0; p < parts && ok; ++p) ok = fwrite(ftxt[p].data(), 1, ftxt[p].size(), f) == ftxt[p].size();
    ok = (fclose(f) == 0) && ok;
    return ok ? fipc::FIPC_OK : fipc::FIPC_ERR_IO;
}

}  // extern "C"
