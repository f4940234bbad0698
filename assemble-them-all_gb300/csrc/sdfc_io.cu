// SDF grid files (host only).
//
// Text: the reference's .sdf cache (BodySDFObj::save_SDF / load_SDF,
// simulation/redmax/Body/BodySDFObj.cpp:86-116; SDFMesh::save_SDF / load_SDF,
// simulation/redmax/Mesh.cpp:103-135): "ni nj nk", min_box, max_box, "dx dy dz" on one line
// each, then one value per line, i fastest, all written by std::ostream's default double
// format (6 significant digits, so the cache is lossy) and read back by operator>>.
//
// Bricks: this library's binary cache of SDFC_STORAGE_F16_BRICKS grids, little-endian:
//   char[8] "SDFCBRK1"; int32 ni, nj, nk, 0; float64 min_box[3], max_box[3], dxyz[3];
//   uint16 codes[nb * 512]; float32 so[2 * nb]        (nb = ceil(ni/8) ceil(nj/8) ceil(nk/8))
// holding exactly what sdfc_f16_brick_encode produced, so a loaded grid uploads without
// re-encoding (sdfc_upload_grid_bricks) and evaluates identically.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "sdfc.h"

namespace {

constexpr char kBrickMagic[8] = {'S', 'D', 'F', 'C', 'B', 'R', 'K', '1'};

bool shape_ok(int ni, int nj, int nk) {
    return ni >= 1 && nj >= 1 && nk >= 1 && (double)ni * nj * nk < 4.0e9;
}

size_t bricks_of(int ni, int nj, int nk) {
    return (size_t)((ni + 7) / 8) * (size_t)((nj + 7) / 8) * (size_t)((nk + 7) / 8);
}

// Whitespace-separated tokens of a whole file, parsed as operator>> would (strtod and strtol
// give the same values as libstdc++'s num_get, which calls them).
struct Tokens {
    std::vector<char> buf;
    size_t pos = 0;
    bool open(const char* path) {
        FILE* f = std::fopen(path, "rb");
        if (!f) return false;
        char chunk[1 << 16];
        size_t r;
        while ((r = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + r);
        std::fclose(f);
        buf.push_back('\0');
        return true;
    }
    const char* next() {
        while (pos < buf.size() && (buf[pos] == ' ' || buf[pos] == '\n' || buf[pos] == '\t' || buf[pos] == '\r'))
            ++pos;
        if (pos >= buf.size() || buf[pos] == '\0') return nullptr;
        return &buf[pos];
    }
    bool read_int(int& v) {
        const char* p = next();
        if (!p) return false;
        char* end = nullptr;
        errno = 0;
        const long x = std::strtol(p, &end, 10);
        if (end == p || errno || x < INT32_MIN || x > INT32_MAX) return false;
        v = (int)x;
        pos += (size_t)(end - p);
        return true;
    }
    bool read_double(double& v) {
        const char* p = next();
        if (!p) return false;
        char* end = nullptr;
        v = std::strtod(p, &end);
        if (end == p) return false;
        pos += (size_t)(end - p);
        return true;
    }
};

}  // namespace

extern "C" {

int sdfc_sdf_save_text(const char* path, const double* values, int ni, int nj, int nk, const double min_box[3],
                       const double max_box[3], const double dxyz[3]) {
    if (!path || !values || !min_box || !max_box || !dxyz || !shape_ok(ni, nj, nk)) return SDFC_ERR_INVALID_ARGUMENT;
    std::ofstream out(path);
    if (!out.good()) return SDFC_ERR_NOT_FOUND;
    out << ni << " " << nj << " " << nk << std::endl;
    out << min_box[0] << " " << min_box[1] << " " << min_box[2] << std::endl;
    out << max_box[0] << " " << max_box[1] << " " << max_box[2] << std::endl;
    out << dxyz[0] << " " << dxyz[1] << " " << dxyz[2] << std::endl;
    const size_t n = (size_t)ni * nj * nk;
    for (size_t i = 0; i < n; ++i) out << values[i] << std::endl;
    out.close();
    return out.fail() ? SDFC_ERR_NOT_FOUND : SDFC_OK;
}

int sdfc_sdf_load_text(const char* path, int shape[3], double min_box[3], double max_box[3], double dxyz[3],
                       double* values, long long capacity) {
    if (!path || !shape || !min_box || !max_box || !dxyz) return SDFC_ERR_INVALID_ARGUMENT;
    Tokens t;
    if (!t.open(path)) return SDFC_ERR_NOT_FOUND;
    int ni, nj, nk;
    if (!t.read_int(ni) || !t.read_int(nj) || !t.read_int(nk) || !shape_ok(ni, nj, nk))
        return SDFC_ERR_INVALID_ARGUMENT;
    double h[9];
    for (double& x : h)
        if (!t.read_double(x)) return SDFC_ERR_INVALID_ARGUMENT;
    shape[0] = ni;
    shape[1] = nj;
    shape[2] = nk;
    for (int a = 0; a < 3; ++a) {
        min_box[a] = h[a];
        max_box[a] = h[3 + a];
        dxyz[a] = h[6 + a];
    }
    if (!values) return SDFC_OK;
    const long long n = (long long)ni * nj * nk;
    if (capacity < n) return SDFC_ERR_CAPACITY;
    for (long long i = 0; i < n; ++i)
        if (!t.read_double(values[i])) return SDFC_ERR_INVALID_ARGUMENT;
    return SDFC_OK;
}

int sdfc_sdf_save_bricks(const char* path, const double* values, int ni, int nj, int nk, const double min_box[3],
                         const double max_box[3], const double dxyz[3]) {
    if (!path || !values || !min_box || !max_box || !dxyz || !shape_ok(ni, nj, nk)) return SDFC_ERR_INVALID_ARGUMENT;
    const size_t nb = bricks_of(ni, nj, nk);
    std::vector<unsigned short> codes(nb * 512);
    std::vector<float> so(2 * nb);
    int rc = sdfc_f16_brick_encode(values, ni, nj, nk, codes.data(), so.data());
    if (rc) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return SDFC_ERR_NOT_FOUND;
    const int32_t hdr[4] = {ni, nj, nk, 0};
    double box[9];
    for (int a = 0; a < 3; ++a) {
        box[a] = min_box[a];
        box[3 + a] = max_box[a];
        box[6 + a] = dxyz[a];
    }
    bool ok = std::fwrite(kBrickMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(hdr), 1, f) == 1 &&
              std::fwrite(box, sizeof(box), 1, f) == 1 &&
              std::fwrite(codes.data(), sizeof(unsigned short), codes.size(), f) == codes.size() &&
              std::fwrite(so.data(), sizeof(float), so.size(), f) == so.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? SDFC_OK : SDFC_ERR_NOT_FOUND;
}

int sdfc_sdf_load_bricks(const char* path, int shape[3], double min_box[3], double max_box[3], double dxyz[3],
                         unsigned short* codes, float* so) {
    if (!path || !shape || !min_box || !max_box || !dxyz) return SDFC_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return SDFC_ERR_NOT_FOUND;
    char magic[8];
    int32_t hdr[4];
    double box[9];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kBrickMagic, 8) == 0 &&
              std::fread(hdr, sizeof(hdr), 1, f) == 1 && std::fread(box, sizeof(box), 1, f) == 1 &&
              shape_ok(hdr[0], hdr[1], hdr[2]);
    if (ok) {
        for (int a = 0; a < 3; ++a) {
            shape[a] = hdr[a];
            min_box[a] = box[a];
            max_box[a] = box[3 + a];
            dxyz[a] = box[6 + a];
        }
        if (codes && so) {
            const size_t nb = bricks_of(hdr[0], hdr[1], hdr[2]);
            ok = std::fread(codes, sizeof(unsigned short), nb * 512, f) == nb * 512 &&
                 std::fread(so, sizeof(float), 2 * nb, f) == 2 * nb;
        }
    }
    std::fclose(f);
    return ok ? SDFC_OK : SDFC_ERR_INVALID_ARGUMENT;
}

}  // extern "C"
