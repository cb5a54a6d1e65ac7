// vtk.cpp — legacy-VTK particle files, the reference's output format.
//
// Reference counterparts: output_fluid_file writes "./result/fluid_t=<step>.vtk" as an ASCII
// UNSTRUCTURED_GRID of POINTS with POINT_DATA "p" (scalar) and "velocity" (vector) in double
// text (src/io/io.cu:154-199); the later version writes the same layout with BINARY
// big-endian floats (opt_src_v3/io/io.cu:121-200).  sph_write_vtk writes either form from
// host arrays in original particle order, adding the particle kind as a third point array
// when it is given.  Host code only; it runs on the caller's thread (a writer thread fed by
// sph_snapshot_begin/wait overlaps it with the GPU).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "sph_gb300.h"

namespace {

uint32_t be32(uint32_t v) {
    return ((v & 0xffu) << 24) | ((v & 0xff00u) << 8) | ((v >> 8) & 0xff00u) | (v >> 24);
}

// n * per values as big-endian 32-bit words
template <class T>
bool put_be(FILE* f, const T* a, long count) {
    static_assert(sizeof(T) == 4, "32-bit values");
    std::vector<uint32_t> buf(4096);
    for (long i = 0; i < count; i += (long)buf.size()) {
        const long m = count - i < (long)buf.size() ? count - i : (long)buf.size();
        for (long k = 0; k < m; k++) {
            uint32_t u;
            std::memcpy(&u, a + i + k, 4);
            buf[k] = be32(u);
        }
        if (std::fwrite(buf.data(), 4, (size_t)m, f) != (size_t)m) return false;
    }
    return true;
}

bool put_text(FILE* f, const float* a, long n, int per) {
    for (long i = 0; i < n; i++) {
        for (int c = 0; c < per; c++)
            if (std::fprintf(f, c ? " %.9g" : "%.9g", (double)a[per * i + c]) < 0) return false;
        if (std::fputc('\n', f) == EOF) return false;
    }
    return true;
}

}  // namespace

extern "C" int sph_write_vtk(const char* path, int n, const float* pos, const float* vel,
                             const float* p, const int* type, int binary) {
    if (!path || n < 0 || (n > 0 && (!pos || !vel || !p))) return SPH_ERR_ARG;
    FILE* f = std::fopen(path, "wb");
    if (!f) return SPH_ERR_ARG;
    bool ok = std::fprintf(f, "# vtk DataFile Version 3.0\nsph data\n%s\nDATASET UNSTRUCTURED_GRID\n"
                              "POINTS %d float\n", binary ? "BINARY" : "ASCII", n) > 0;
    ok = ok && (binary ? put_be(f, pos, 3L * n) : put_text(f, pos, n, 3));
    ok = ok && std::fprintf(f, "%sPOINT_DATA %d\nSCALARS p float 1\nLOOKUP_TABLE DEFAULT\n",
                            binary ? "\n" : "", n) > 0;
    ok = ok && (binary ? put_be(f, p, n) : put_text(f, p, n, 1));
    ok = ok && std::fprintf(f, "%sVECTORS velocity float\n", binary ? "\n" : "") > 0;
    ok = ok && (binary ? put_be(f, vel, 3L * n) : put_text(f, vel, n, 3));
    if (type) {
        ok = ok && std::fprintf(f, "%sSCALARS type int 1\nLOOKUP_TABLE DEFAULT\n",
                                binary ? "\n" : "") > 0;
        if (binary) {
            ok = ok && put_be(f, type, n);
        } else {
            for (long i = 0; ok && i < n; i++) ok = std::fprintf(f, "%d\n", type[i]) > 0;
        }
    }
    if (binary) ok = ok && std::fputc('\n', f) != EOF;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? SPH_OK : SPH_ERR_ARG;
}
