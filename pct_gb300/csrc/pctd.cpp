/*
 * PCTD version-0 proton history files: reader and writer.
 *
 * Layout, as count_histories_v0 and read_data_chunk_v02 read it
 * (src/pCT_Reconstruction_Data_Segments.cu:997-1097, 1769-1933), little endian:
 *   char[4] "PCTD", int32 version (0), int32 number of histories N,
 *   float32 projection angle [deg], float32 beam energy [MeV],
 *   int32 generation date, int32 pre-process date,
 *   three strings (int32 length + bytes): phantom name, data source, prepared by,
 *   float32[N] x 13: t0..t3, v0..v3, u0..u3, WEPL (mm), one array after another.
 * The reader checks every length against the file size and fails with
 * PCT_ERR_IO on a malformed file (the reference reads whatever is there).
 */
#include <cstdio>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>
#include "pct_internal.h"

#define PCT_TRY(call)                         \
    do {                                      \
        pct_status s_ = (call);               \
        if (s_ != PCT_OK) return s_;          \
    } while (0)

namespace {

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

bool read_exact(FILE* f, void* dst, size_t n) { return fread(dst, 1, n, f) == n; }

/* Host byte order is little endian on every supported host (x86-64, aarch64). */
pct_status read_header(FILE* f, const char* path, int64_t file_size, int32_t* n, float* angle, float* energy,
                       int64_t* data_offset) {
    char magic[4];
    int32_t version = 0, count = 0, dates[2];
    float ae[2];
    if (!read_exact(f, magic, 4) || memcmp(magic, "PCTD", 4) != 0)
        return pct_fail(PCT_ERR_IO, "%s: not a PCTD file", path);
    if (!read_exact(f, &version, 4) || !read_exact(f, &count, 4) || !read_exact(f, ae, 8) || !read_exact(f, dates, 8))
        return pct_fail(PCT_ERR_IO, "%s: truncated header", path);
    if (version != 0) return pct_fail(PCT_ERR_IO, "%s: PCTD version %d is not supported", path, version);
    if (count < 0) return pct_fail(PCT_ERR_IO, "%s: negative history count", path);
    int64_t off = 28;
    for (int s = 0; s < 3; ++s) {
        int32_t len = 0;
        if (!read_exact(f, &len, 4)) return pct_fail(PCT_ERR_IO, "%s: truncated header", path);
        if (len < 0 || off + 4 + len > file_size) return pct_fail(PCT_ERR_IO, "%s: bad string length", path);
        if (fseek(f, len, SEEK_CUR) != 0) return pct_fail(PCT_ERR_IO, "%s: seek failed", path);
        off += 4 + len;
    }
    if (off + 52 * (int64_t)count > file_size)
        return pct_fail(PCT_ERR_IO, "%s: truncated history data (%lld of %lld bytes)", path,
                        (long long)(file_size - off), (long long)(52 * (int64_t)count));
    *n = count;
    if (angle) *angle = ae[0];
    if (energy) *energy = ae[1];
    *data_offset = off;
    return PCT_OK;
}

pct_status open_file(const char* path, File& fh, int64_t* size) {
    if (!path) return pct_fail(PCT_ERR_ARGUMENT, "PCTD: null path");
    fh.f = fopen(path, "rb");
    if (!fh.f) return pct_fail(PCT_ERR_IO, "%s: cannot open", path);
    if (fseek(fh.f, 0, SEEK_END) != 0) return pct_fail(PCT_ERR_IO, "%s: seek failed", path);
    *size = (int64_t)ftell(fh.f);
    rewind(fh.f);
    return PCT_OK;
}

}  // namespace

extern "C" pct_status pct_pctd_info(const char* path, int64_t* num_histories, float* projection_angle,
                                    float* beam_energy) {
    if (!num_histories) return pct_fail(PCT_ERR_ARGUMENT, "pct_pctd_info: null argument");
    File fh;
    int64_t size = 0, off = 0;
    PCT_TRY(open_file(path, fh, &size));
    int32_t n = 0;
    PCT_TRY(read_header(fh.f, path, size, &n, projection_angle, beam_energy, &off));
    *num_histories = n;
    return PCT_OK;
}

extern "C" pct_status pct_pctd_read(const char* path, float* const data13[13], int64_t capacity, int64_t* n_out,
                                    float* projection_angle) {
    if (!data13 || !n_out) return pct_fail(PCT_ERR_ARGUMENT, "pct_pctd_read: null argument");
    File fh;
    int64_t size = 0, off = 0;
    PCT_TRY(open_file(path, fh, &size));
    int32_t n = 0;
    PCT_TRY(read_header(fh.f, path, size, &n, projection_angle, nullptr, &off));
    if (n > capacity)
        return pct_fail(PCT_ERR_OVERFLOW, "%s: %d histories exceed the capacity %lld", path, n, (long long)capacity);
    for (int k = 0; k < 13; ++k) {
        if (!data13[k]) return pct_fail(PCT_ERR_ARGUMENT, "pct_pctd_read: null array %d", k);
        if (n > 0 && !read_exact(fh.f, data13[k], sizeof(float) * (size_t)n))
            return pct_fail(PCT_ERR_IO, "%s: read failed", path);
    }
    *n_out = n;
    return PCT_OK;
}

extern "C" pct_status pct_pctd_write(const char* path, const float* const data13[13], int64_t n,
                                     float projection_angle, float beam_energy) {
    if (!path || !data13 || n < 0 || n > 0x7fffffff) return pct_fail(PCT_ERR_ARGUMENT, "pct_pctd_write: bad argument");
    FILE* f = fopen(path, "wb");
    if (!f) return pct_fail(PCT_ERR_IO, "%s: cannot create", path);
    File fh;
    fh.f = f;
    const int32_t version = 0, count = (int32_t)n, dates[2] = {0, 0};
    const float ae[2] = {projection_angle, beam_energy};
    const char* strings[3] = {"synthetic", "pct_gb300 generator", "pct_gb300"};
    bool ok = fwrite("PCTD", 1, 4, f) == 4 && fwrite(&version, 4, 1, f) == 1 && fwrite(&count, 4, 1, f) == 1 &&
              fwrite(ae, 4, 2, f) == 2 && fwrite(dates, 4, 2, f) == 2;
    for (int s = 0; ok && s < 3; ++s) {
        int32_t len = (int32_t)strlen(strings[s]);
        ok = fwrite(&len, 4, 1, f) == 1 && fwrite(strings[s], 1, (size_t)len, f) == (size_t)len;
    }
    for (int k = 0; ok && k < 13; ++k) {
        if (!data13[k]) return pct_fail(PCT_ERR_ARGUMENT, "pct_pctd_write: null array %d", k);
        ok = n == 0 || fwrite(data13[k], sizeof(float), (size_t)n, f) == (size_t)n;
    }
    if (!ok) return pct_fail(PCT_ERR_IO, "%s: write failed", path);
    return PCT_OK;
}

/* Page-locked staging for the file uploads (freed on scope exit); empty when
 * the allocation fails, and pageable memory is used instead. */
struct Pinned {
    float* p = nullptr;
    explicit Pinned(size_t n) {
        if (cudaMallocHost(reinterpret_cast<void**>(&p), n * sizeof(float)) != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
        }
    }
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

/* Reads each file and uploads it as one chunk (the histories of one file share
 * the header's projection angle), like the read_data_chunk / hull_detection
 * loop of the reference driver (.cu:97-100).  The files are read into one
 * page-locked buffer sized for the largest, so that the uploads run at full
 * host-link speed; pct_process_chunk returns after the chunk's uploads have
 * completed (its compaction synchronises the stream), so the buffer is reused. */
extern "C" pct_status pct_process_pctd_files(pct_ctx* ctx, const char* const* paths, int num_files) {
    if (!ctx || (!paths && num_files > 0) || num_files < 0)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_process_pctd_files: bad argument");
    int64_t nmax = 1;
    for (int i = 0; i < num_files; ++i) {
        int64_t n = 0;
        PCT_TRY(pct_pctd_info(paths[i], &n, nullptr, nullptr));
        nmax = n > nmax ? n : nmax;
    }
    const size_t need = (size_t)14 * (size_t)nmax; /* 13 arrays and the angles */
    Pinned pinned(need);
    std::vector<float> pageable;
    float* base = pinned.p;
    if (!base) {
        pageable.resize(need);
        base = pageable.data();
    }
    for (int i = 0; i < num_files; ++i) {
        int64_t n = 0;
        float angle = 0.0f;
        PCT_TRY(pct_pctd_info(paths[i], &n, &angle, nullptr));
        float* d13[13];
        for (int k = 0; k < 13; ++k) d13[k] = base + (size_t)k * (size_t)nmax;
        int64_t got = 0;
        PCT_TRY(pct_pctd_read(paths[i], d13, nmax, &got, &angle));
        if (got == 0) continue;
        float* ang = base + (size_t)13 * (size_t)nmax;
        for (int64_t j = 0; j < got; ++j) ang[j] = angle;
        const float* c13[13];
        for (int k = 0; k < 13; ++k) c13[k] = d13[k];
        PCT_TRY(pct_process_chunk(ctx, c13, ang, got, 0));
    }
    return PCT_OK;
}
