// Gauge configuration files in the reference's two formats.
//
//   "SWNG" (save_gauge / load_gauge, reference src/hmc_forces.cpp:18-62): the
//   32-byte GaugeHeader {uint32 magic = 0x53574E47, uint32 L, double beta,
//   double mass, double avg_plaq} (src/hmc.h:19-25), then U[0][s] and U[1][s]
//   for s = x + L y as complex128.  Loading divides every link by its modulus.
//   raw (GaugeField::save / load, src/gauge.h:38-57): int32 V, then the links.
//
// Bytes are written and read little-endian explicitly (the reference writes
// its in-memory structs, which are little-endian on x86-64 and AArch64), so
// files are byte-identical to the reference's.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/smg_gpu.h"

namespace {

constexpr uint32_t kMagic = 0x53574E47u;

void put_u32(unsigned char* p, uint32_t v) {
    for (int i = 0; i < 4; ++i) p[i] = (unsigned char)((v >> (8 * i)) & 0xFFu);
}
uint32_t get_u32(const unsigned char* p) {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)p[i] << (8 * i);
    return v;
}
void put_f64(unsigned char* p, double d) {
    uint64_t v;
    std::memcpy(&v, &d, 8);
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char)((v >> (8 * i)) & 0xFFu);
}
double get_f64(const unsigned char* p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)p[i] << (8 * i);
    double d;
    std::memcpy(&d, &v, 8);
    return d;
}

struct File {
    FILE* f = nullptr;
    File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

smg_status write_links(FILE* f, int64_t n_doubles, const double* U) {
    std::vector<unsigned char> buf(8 * 4096);
    for (int64_t i = 0; i < n_doubles; i += 4096) {
        const int64_t c = n_doubles - i < 4096 ? n_doubles - i : 4096;
        for (int64_t j = 0; j < c; ++j) put_f64(buf.data() + 8 * j, U[i + j]);
        if (std::fwrite(buf.data(), 8, (size_t)c, f) != (size_t)c) return SMG_IO_ERROR;
    }
    return SMG_OK;
}

smg_status read_links(FILE* f, int64_t n_doubles, double* U) {
    std::vector<unsigned char> buf(8 * 4096);
    for (int64_t i = 0; i < n_doubles; i += 4096) {
        const int64_t c = n_doubles - i < 4096 ? n_doubles - i : 4096;
        if (std::fread(buf.data(), 8, (size_t)c, f) != (size_t)c) return SMG_IO_ERROR;
        for (int64_t j = 0; j < c; ++j) U[i + j] = get_f64(buf.data() + 8 * j);
    }
    return SMG_OK;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_host_gauge_write_swng(const char* path, int L, const double* U, double beta, double mass,
                                             double avg_plaq) {
    if (!path || !U || L < 2) return SMG_BAD_ARG;
    File fl(path, "wb");
    if (!fl.f) return SMG_IO_ERROR;
    unsigned char h[32];
    put_u32(h, kMagic);
    put_u32(h + 4, (uint32_t)L);
    put_f64(h + 8, beta);
    put_f64(h + 16, mass);
    put_f64(h + 24, avg_plaq);
    if (std::fwrite(h, 1, 32, fl.f) != 32) return SMG_IO_ERROR;
    return write_links(fl.f, (int64_t)4 * L * L, U);
}

SMG_API smg_status smg_host_gauge_read_swng(const char* path, int L_expected, smg_gauge_header* hdr, double* U) {
    if (!path || !hdr) return SMG_BAD_ARG;
    File fl(path, "rb");
    if (!fl.f) return SMG_IO_ERROR;
    unsigned char h[32];
    if (std::fread(h, 1, 32, fl.f) != 32) return SMG_IO_ERROR;
    hdr->magic = get_u32(h);
    hdr->L = get_u32(h + 4);
    hdr->beta = get_f64(h + 8);
    hdr->mass = get_f64(h + 16);
    hdr->avg_plaq = get_f64(h + 24);
    if (hdr->magic != kMagic) return SMG_BAD_ARG;              // "Bad magic number"
    if (L_expected > 0 && (int)hdr->L != L_expected) return SMG_BAD_ARG;  // "Lattice size mismatch"
    if (!U) return SMG_OK;
    // the links are written only when the caller stated the size its buffer was made for: an L taken
    // from the file alone could overrun it
    if (L_expected <= 0) return SMG_BAD_ARG;
    if (hdr->L < 2 || hdr->L > 65536) return SMG_BAD_ARG;
    const int64_t n = (int64_t)4 * hdr->L * hdr->L;
    if (read_links(fl.f, n, U) != SMG_OK) return SMG_IO_ERROR;
    for (int64_t i = 0; i < n; i += 2) {  // U /= |U| (hmc_forces.cpp:56-59)
        const double a = std::hypot(U[i], U[i + 1]);
        U[i] /= a;
        U[i + 1] /= a;
    }
    return SMG_OK;
}

SMG_API smg_status smg_host_gauge_write_raw(const char* path, int L, const double* U) {
    if (!path || !U || L < 2) return SMG_BAD_ARG;
    File fl(path, "wb");
    if (!fl.f) return SMG_IO_ERROR;
    unsigned char h[4];
    put_u32(h, (uint32_t)(L * L));
    if (std::fwrite(h, 1, 4, fl.f) != 4) return SMG_IO_ERROR;
    return write_links(fl.f, (int64_t)4 * L * L, U);
}

SMG_API smg_status smg_host_gauge_read_raw(const char* path, int L, double* U) {
    if (!path || !U || L < 2) return SMG_BAD_ARG;
    File fl(path, "rb");
    if (!fl.f) return SMG_IO_ERROR;
    unsigned char h[4];
    if (std::fread(h, 1, 4, fl.f) != 4) return SMG_IO_ERROR;
    if ((int64_t)(int32_t)get_u32(h) != (int64_t)L * L) return SMG_BAD_ARG;  // V mismatch (gauge.h:52)
    return read_links(fl.f, (int64_t)4 * L * L, U);
}

SMG_API smg_status smg_gauge_save(smg_gauge* g, double beta, double mass, const char* path) {
    if (!g || !path) return SMG_BAD_ARG;
    const int L = smg_gauge_L(g);
    std::vector<double> U((size_t)4 * L * L);
    smg_status s = smg_gauge_get(g, U.data());
    if (s != SMG_OK) return s;
    double plaq = 0;
    s = smg_gauge_avg_plaq(g, &plaq);
    if (s != SMG_OK) return s;
    return smg_host_gauge_write_swng(path, L, U.data(), beta, mass, plaq);
}

SMG_API smg_status smg_gauge_load(smg_gauge* g, const char* path, smg_gauge_header* hdr) {
    if (!g || !path) return SMG_BAD_ARG;
    const int L = smg_gauge_L(g);
    std::vector<double> U((size_t)4 * L * L);
    smg_gauge_header h{};
    smg_status s = smg_host_gauge_read_swng(path, L, &h, U.data());
    if (s != SMG_OK) return s;
    if (hdr) *hdr = h;
    return smg_gauge_set(g, U.data());
}

}  // extern "C"
