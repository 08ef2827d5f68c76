// Seismic Unix trace files on the host, in place of the reference's Fortran
// stream reads and its suaddhead/sushw shell pipeline.
//
//   fwi_su_read   get_shot_data (get_mcs_data.f90:167-207) and the per-OBS read
//                 of get_obs_data (get_was_data.f90:241-288): trace j
//                 (0-based) starts at byte j*(240 + 4*nt); its nt samples
//                 follow the 240-byte header; the file's byte order is given
//                 (the reference's endianness_data, get_mcs_data.f90:317-323).
//   fwi_su_write  write_new_data (auxiliar.f90:433-531) after its resampling:
//                 the traces with SU headers as `suaddhead ns= | sushw key=dt
//                 a=` produce them (Seismic Unix, CWP; its documentation of
//                 suaddhead: trace counters tracl and tracr, trace
//                 identification trid = 1 for a live seismic trace, and ns;
//                 sushw then sets dt): tracl (bytes 0-3) and tracr (4-7) the
//                 1-based trace number, trid (28-29) 1, ns (114-115), dt
//                 (116-117, microseconds); every other header word is 0.
//   fwi_su_supershot  get_obs_data (get_was_data.f90:241-288): the traces of
//                 several OBS files summed with their coding factors into one
//                 gather, raw_data = raw_data + Coding(k)*data in FP32.
//   fwi_su_info   ns and dt from the first header and the trace count from
//                 the file size.
//   fwi_read_nav  the navigation lists (read_nav_shot_mcs, get_mcs_data.f90:
//                 88-117, with the line count of :228-245; read_nav_shot_was,
//                 get_was_data.f90:148-164; read_nav_obs, :196-207): one
//                 record per line, an integer (shot or OBS number) and two
//                 reals (x and water depth, or x and OBS depth), read
//                 list-directed (blanks or commas between values).
//
// Byte order: SU files are written in the host's order by the SU tools;
// big_endian = 1 reads/writes big-endian files on any host.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fwi_gb300.h"

namespace fwi {
int prep_fail(int code, const std::string& msg);  // fwi_host.cu
}

namespace {

constexpr int SU_HEADER = 240;

bool host_big_endian() {
    const uint16_t one = 1;
    unsigned char b[2];
    std::memcpy(b, &one, 2);
    return b[0] == 0;
}

void swap_bytes(void* p, size_t n, size_t width) {
    unsigned char* c = static_cast<unsigned char*>(p);
    for (size_t i = 0; i < n; ++i, c += width)
        for (size_t k = 0; k < width / 2; ++k) {
            const unsigned char t = c[k];
            c[k] = c[width - 1 - k];
            c[width - 1 - k] = t;
        }
}

struct File {
    FILE* f = nullptr;
    explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

uint16_t get_u16(const unsigned char* h, int off, bool swap) {
    uint16_t v;
    std::memcpy(&v, h + off, 2);
    if (swap) swap_bytes(&v, 1, 2);
    return v;
}
void put_u16(unsigned char* h, int off, uint16_t v, bool swap) {
    if (swap) swap_bytes(&v, 1, 2);
    std::memcpy(h + off, &v, 2);
}
void put_i32(unsigned char* h, int off, int32_t v, bool swap) {
    if (swap) swap_bytes(&v, 1, 4);
    std::memcpy(h + off, &v, 4);
}

}  // namespace

extern "C" {

int fwi_su_info(const char* path, int big_endian, int* ns, float* dt, int* ntraces) {
    if (!path || !ns || !dt || !ntraces) return fwi::prep_fail(FWI_ERR_ARG, "null argument");
    File fh(path, "rb");
    if (!fh.f) return fwi::prep_fail(FWI_ERR_ARG, std::string("cannot open ") + path);
    unsigned char h[SU_HEADER];
    if (std::fread(h, 1, SU_HEADER, fh.f) != SU_HEADER)
        return fwi::prep_fail(FWI_ERR_ARG, std::string(path) + ": shorter than one SU header");
    const bool swap = (big_endian != 0) != host_big_endian();
    *ns = get_u16(h, 114, swap);
    *dt = (float)get_u16(h, 116, swap) * 1e-6f;
    std::fseek(fh.f, 0, SEEK_END);
    const long size = std::ftell(fh.f);
    const long tr = SU_HEADER + 4L * (*ns);
    *ntraces = (*ns > 0) ? (int)(size / tr) : 0;
    return FWI_OK;
}

int fwi_su_read(const char* path, int nt, int ntr, int big_endian, float* out) {
    if (!path || !out) return fwi::prep_fail(FWI_ERR_ARG, "null argument");
    if (nt < 1 || ntr < 0) return fwi::prep_fail(FWI_ERR_ARG, "nt must be >= 1 and ntr >= 0");
    File fh(path, "rb");
    if (!fh.f) return fwi::prep_fail(FWI_ERR_ARG, std::string("cannot open ") + path);
    const bool swap = (big_endian != 0) != host_big_endian();
    const long stride = SU_HEADER + 4L * nt;
    for (int j = 0; j < ntr; ++j) {
        if (std::fseek(fh.f, (long)j * stride + SU_HEADER, SEEK_SET) != 0 ||
            std::fread(out + (size_t)j * nt, 4, (size_t)nt, fh.f) != (size_t)nt)
            return fwi::prep_fail(FWI_ERR_ARG, std::string(path) + ": fewer than " + std::to_string(ntr) +
                                                   " traces of " + std::to_string(nt) + " samples");
        if (swap) swap_bytes(out + (size_t)j * nt, (size_t)nt, 4);
    }
    return FWI_OK;
}

int fwi_su_write(const char* path, const float* data, int nt, int ntr, float dt, int big_endian) {
    if (!path || (!data && ntr > 0)) return fwi::prep_fail(FWI_ERR_ARG, "null argument");
    if (nt < 1 || nt > 65535 || ntr < 0) return fwi::prep_fail(FWI_ERR_ARG, "nt must be in 1..65535 (SU ns)");
    const double us = (double)dt * 1e6;
    if (!(us >= 0.0) || us > 65535.0) return fwi::prep_fail(FWI_ERR_ARG, "dt out of the SU header's range");
    File fh(path, "wb");
    if (!fh.f) return fwi::prep_fail(FWI_ERR_ARG, std::string("cannot create ") + path);
    const bool swap = (big_endian != 0) != host_big_endian();
    std::vector<float> tr(nt);
    for (int j = 0; j < ntr; ++j) {
        unsigned char h[SU_HEADER] = {0};
        put_i32(h, 0, j + 1, swap);                     // tracl
        put_i32(h, 4, j + 1, swap);                     // tracr
        put_u16(h, 28, 1, swap);                        // trid: live seismic trace
        put_u16(h, 114, (uint16_t)nt, swap);            // ns
        put_u16(h, 116, (uint16_t)(int)(dt * 1e6f), swap);  // dt (us), the reference's dt_head = dt2*1e6
        std::memcpy(tr.data(), data + (size_t)j * nt, 4 * (size_t)nt);
        if (swap) swap_bytes(tr.data(), (size_t)nt, 4);
        if (std::fwrite(h, 1, SU_HEADER, fh.f) != SU_HEADER || std::fwrite(tr.data(), 4, (size_t)nt, fh.f) != (size_t)nt)
            return fwi::prep_fail(FWI_ERR_ARG, std::string(path) + ": write failed");
    }
    return FWI_OK;
}

int fwi_su_supershot(const char* const* paths, int nsrc, const float* coding, int nt, int ntr, int big_endian,
                     float* raw_data) {
    if (!paths || !coding || !raw_data || nsrc < 0) return fwi::prep_fail(FWI_ERR_ARG, "null argument");
    if (nt < 1 || ntr < 0) return fwi::prep_fail(FWI_ERR_ARG, "nt must be >= 1 and ntr >= 0");
    const size_t n = (size_t)nt * ntr;
    for (size_t i = 0; i < n; ++i) raw_data[i] = 0.f;  // raw_Data=0. (:265)
    std::vector<float> tmp(n);
    for (int k = 0; k < nsrc; ++k) {
        if (!paths[k]) return fwi::prep_fail(FWI_ERR_ARG, "null path");
        const int rc = fwi_su_read(paths[k], nt, ntr, big_endian, tmp.data());
        if (rc != FWI_OK) return rc;
        const float c = coding[k];
        for (size_t i = 0; i < n; ++i) raw_data[i] = raw_data[i] + c * tmp[i];  // :282
    }
    return FWI_OK;
}

int fwi_read_nav(const char* path, int max_records, int* shot_id, float* xs, float* bat, int* nrecords) {
    if (!path || !nrecords || (max_records > 0 && (!shot_id || !xs || !bat)))
        return fwi::prep_fail(FWI_ERR_ARG, "null argument");
    File fh(path, "r");
    if (!fh.f) return fwi::prep_fail(FWI_ERR_ARG, std::string("cannot open ") + path);
    char line[4096];
    int n = 0, lineno = 0;
    while (std::fgets(line, sizeof line, fh.f)) {
        ++lineno;
        for (char* c = line; *c; ++c)
            if (*c == ',') *c = ' ';
        char* p = line;
        while (*p == ' ' || *p == '\t') ++p;
        if (*p == '\n' || *p == '\r' || *p == 0) continue;  // blank line
        char* e1;
        const long id = std::strtol(p, &e1, 10);
        char* e2;
        const float x = std::strtof(e1, &e2);
        char* e3;
        const float b = std::strtof(e2, &e3);
        if (e1 == p || e2 == e1 || e3 == e2)
            return fwi::prep_fail(FWI_ERR_ARG, std::string(path) + ":" + std::to_string(lineno) +
                                                   ": expected shot number, x and depth");
        if (n < max_records) {
            shot_id[n] = (int)id;
            xs[n] = x;
            bat[n] = b;
        }
        ++n;
    }
    *nrecords = n;
    return FWI_OK;
}

}  // extern "C"
