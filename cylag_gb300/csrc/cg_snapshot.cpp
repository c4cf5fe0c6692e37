// cg_snapshot.cpp -- particle snapshots in CyLag's text and VTK formats.
//
// Host code.  The reference formats every particle with Python's str.format
// (cylag/io/writer_txt.pyx:25-180, cylag/io/writer_vtk.pyx:25-304), one
// write per value; here each snapshot is formatted in parallel chunks (one
// per host thread) into memory and written once, byte-identical to the
// reference's files:
//   '{:16d}'  -> "%16d";  '{:.16e}', '{:.8e}', '{:.8f}' -> the same printf
//   conversions (both correctly rounded);  '{}' of a float -> Python's repr
//   (shortest round-trip digits, fixed notation for decimal exponents in
//   (-4, 16], else d.ddde+XX; ".0" after an integral fixed value).
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cylag_gpu.h"

namespace {

void put_fmt(std::string& s, const char* fmt, double v) {
    char b[64];
    int k = std::snprintf(b, sizeof b, fmt, v);
    s.append(b, k);
}

void put_int(std::string& s, const char* fmt, long long v) {
    char b[32];
    int k = std::snprintf(b, sizeof b, fmt, v);
    s.append(b, k);
}

// Python repr of a double (float_repr_style 'short')
void put_repr(std::string& s, double v) {
    if (std::isnan(v)) { s += "nan"; return; }
    if (std::isinf(v)) { s += v < 0 ? "-inf" : "inf"; return; }
    if (v == 0.) { s += std::signbit(v) ? "-0.0" : "0.0"; return; }
    char b[64];
    auto r = std::to_chars(b, b + sizeof b - 1, v, std::chars_format::scientific);
    *r.ptr = '\0';
    // b = [-]d[.ddd]e(+|-)XX : the shortest round-trip digits
    const char* p = b;
    const char* end = r.ptr;
    bool neg = *p == '-';
    if (neg) ++p;
    char digits[32];
    int nd = 0;
    const char* q = p;
    for (; q < end && *q != 'e'; ++q)
        if (*q != '.') digits[nd++] = *q;
    int e10 = std::atoi(q + 1);
    const int decpt = e10 + 1;    // value = 0.digits x 10^decpt
    if (neg) s += '-';
    if (decpt <= -4 || decpt > 16) {
        s += digits[0];
        if (nd > 1) {
            s += '.';
            s.append(digits + 1, nd - 1);
        }
        char eb[8];
        int k = std::snprintf(eb, sizeof eb, "e%c%02d", e10 < 0 ? '-' : '+', std::abs(e10));
        s.append(eb, k);
    } else if (decpt <= 0) {
        s += "0.";
        s.append(-decpt, '0');
        s.append(digits, nd);
    } else if (decpt < nd) {
        s.append(digits, decpt);
        s += '.';
        s.append(digits + decpt, nd - decpt);
    } else {
        s.append(digits, nd);
        s.append(decpt - nd, '0');
        s += ".0";
    }
}

struct Snap {
    int dim, model;
    int n;
    const int32_t* tri;
    const int32_t* tag;
    const double* pos;
    const double* vel;
    const double* fvs;
    const double* diam;
    const double* depth;
};

// chunk boundaries over [0, n) and the active indices of each
template <typename F>
std::string parallel_format(int n, F&& fmt_range) {
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 20000) nt = 1;
    std::vector<std::string> part(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) {
        int a = (int)((long long)n * t / nt), b = (int)((long long)n * (t + 1) / nt);
        if (nt == 1) fmt_range(a, b, part[t]);
        else th.emplace_back([&, a, b, t] { fmt_range(a, b, part[t]); });
    }
    for (auto& x : th) x.join();
    size_t tot = 0;
    for (auto& x : part) tot += x.size();
    std::string out;
    out.reserve(tot);
    for (auto& x : part) out += x;
    return out;
}

int write_all(const char* path, const char* mode, const std::string& a) {
    FILE* f = std::fopen(path, mode);
    if (!f) return CG_EINVAL;
    size_t w = std::fwrite(a.data(), 1, a.size(), f);
    int rc = std::fclose(f);
    return (w == a.size() && rc == 0) ? CG_OK : CG_EINVAL;
}

int count_active(const Snap& s) {
    int na = 0;
    for (int i = 0; i < s.n; ++i) na += s.tri[i] != -1;
    return na;
}

}  // namespace

extern "C" {

int cg_snapshot_txt(const char* path, int32_t dim, int32_t model, double time, int64_t iteration,
                    int32_t n, const int32_t* tri, const int32_t* tag, const double* pos,
                    const double* vel, const double* fvs, const double* diameter,
                    const double* depth) {
    if (!path || (dim != 2 && dim != 3) || n < 0 || (n > 0 && (!tri || !tag || !pos || !vel)) ||
        (model >= 2 && n > 0 && !fvs))
        return CG_EINVAL;
    Snap s{dim, model, n, tri, tag, pos, vel, fvs, diameter, depth};
    std::string head;
    put_fmt(head, "Time = %.8f, ", time);
    put_int(head, "Iter = %16lld, ", (long long)iteration);
    put_int(head, "Npart = %16lld\n", count_active(s));
    std::string body = parallel_format(n, [&](int a, int b, std::string& o) {
        o.reserve((size_t)(b - a) * (dim == 2 ? 150 : 180));
        for (int j = a; j < b; ++j) {
            if (s.tri[j] == -1) continue;
            put_int(o, "%16lld, ", s.tag[j]);
            const double* x = s.pos + (size_t)j * dim;
            const double* u = s.vel + (size_t)j * dim;
            put_fmt(o, "%.16e, ", x[0]);
            put_fmt(o, "%.16e, ", x[1]);
            if (dim == 3) put_fmt(o, "%.16e, ", x[2]);
            else o += "0, ";
            put_fmt(o, "%.8e, ", u[0]);
            put_fmt(o, "%.8e, ", u[1]);
            if (dim == 3) put_fmt(o, "%.8e, ", u[2]);
            else o += "0, ";
            if (s.model >= 2) {
                const double* w = s.fvs + (size_t)j * dim;
                put_fmt(o, "%.8e, ", w[0]);
                put_fmt(o, "%.8e, ", w[1]);
                if (dim == 3) put_fmt(o, "%.8e, ", w[2]);
                else o += "0, ";
            }
            if (s.diam) put_fmt(o, "%.8e, ", s.diam[j]);
            if (s.depth) put_fmt(o, "%.8e, ", s.depth[j]);
            o += '\n';
        }
    });
    return write_all(path, "ab", head + body);
}

int cg_snapshot_vtk(const char* path, int32_t dim, int32_t model, double time, int64_t iteration,
                    int32_t n, const int32_t* tri, const int32_t* tag, const double* pos,
                    const double* vel, const double* fvs, const double* diameter,
                    const double* depth) {
    if (!path || (dim != 2 && dim != 3) || n < 0 || (n > 0 && (!tri || !tag || !pos || !vel)) ||
        (model >= 2 && n > 0 && !fvs))
        return CG_EINVAL;
    Snap s{dim, model, n, tri, tag, pos, vel, fvs, diameter, depth};
    const int na = count_active(s);
    // one pass per section, each section formatted in parallel
    auto section = [&](auto&& line) {
        return parallel_format(n, [&](int a, int b, std::string& o) {
            for (int j = a; j < b; ++j)
                if (s.tri[j] != -1) line(j, o);
        });
    };
    auto vec3 = [&](const double* v, int j, std::string& o) {
        put_repr(o, v[(size_t)j * dim]);
        o += ' ';
        put_repr(o, v[(size_t)j * dim + 1]);
        o += ' ';
        put_repr(o, dim == 3 ? v[(size_t)j * dim + 2] : 0.);
        o += '\n';
    };
    std::string out;
    out += "# vtk DataFile Version 2.0\n";
    out += dim == 2 ? "particle positions (Points 2D)\n" : "particle positions (Points 3D)\n";
    out += "ASCII\n";
    out += "DATASET UNSTRUCTURED_GRID\n";
    out += "FIELD FIELDDATA 2\n";
    out += "TIME 1 1 DOUBLE\n";
    put_repr(out, time);
    out += "\nCYCLE 1 1 INT\n";
    put_int(out, "%lld\n", (long long)iteration);
    put_int(out, "POINTS %lld FLOAT\n", na);
    out += section([&](int j, std::string& o) { vec3(s.pos, j, o); });
    char b[96];
    std::snprintf(b, sizeof b, "CELLS %d %lld\n", na, 2LL * na);
    out += b;
    {
        std::string c;
        c.reserve((size_t)na * 10);
        for (int k = 0; k < na; ++k) put_int(c, "1 %lld\n", k);
        out += c;
    }
    put_int(out, "CELL_TYPES %lld\n", na);
    for (int k = 0; k < na; ++k) out += "1\n";
    put_int(out, "POINT_DATA %lld\n", na);
    out += "SCALARS Index INT\nLOOKUP_TABLE default\n";
    out += section([&](int j, std::string& o) { put_int(o, "%lld\n", j); });
    out += "SCALARS tag INT\nLOOKUP_TABLE default\n";
    out += section([&](int j, std::string& o) { put_int(o, "%lld\n", s.tag[j]); });
    if (dim == 3) {
        out += "SCALARS elevation FLOAT\nLOOKUP_TABLE default\n";
        out += section([&](int j, std::string& o) {
            put_repr(o, s.pos[(size_t)j * 3 + 2]);
            o += '\n';
        });
    }
    out += "VECTORS velocity FLOAT\n";
    out += section([&](int j, std::string& o) { vec3(s.vel, j, o); });
    if (s.diam) {
        out += "SCALARS diameter FLOAT\nLOOKUP_TABLE default\n";
        out += section([&](int j, std::string& o) {
            put_repr(o, s.diam[j]);
            o += '\n';
        });
    }
    if (model >= 2) {
        out += "VECTORS fluid_velocity_seen FLOAT\n";
        out += section([&](int j, std::string& o) { vec3(s.fvs, j, o); });
    }
    if (s.depth) {
        out += "SCALARS depth FLOAT\nLOOKUP_TABLE default\n";
        out += section([&](int j, std::string& o) {
            put_repr(o, s.depth[j]);
            o += '\n';
        });
    }
    return write_all(path, "wb", out);
}

}  // extern "C"
