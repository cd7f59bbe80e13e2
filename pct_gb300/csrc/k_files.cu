/*
 * MLP endpoint and path files, and binary image checkpoints.
 *
 * Endpoints: the layout of write_MLP_endpoints / read_MLP_endpoints
 * (src/pCT_Reconstruction_Data_Segments.cu:4684-4745): uint32 N, then N-element
 * arrays int32 voxel_x, voxel_y, voxel_z (the first MLP voxel), int32 bin,
 * float WEPL, x/y/z entry, x/y/z exit, xy/xz entry angle, xy/xz exit angle.
 * Paths: the file the reference's CPU reconstruction writes (.cu:7478-7493):
 * an ASCII line "<N>\n", then per history uint32 count and count uint32 voxel
 * indices (write_MLP_path, .cu:4746).  The reader takes exactly one newline
 * after the count (the reference's fscanf("%u\n") also swallows following
 * bytes that look like white space).  Images: NUM_VOXELS float32, x fastest
 * (the reference writes its iterates as text, .cu:8092-8134).
 */
#include <cstdio>
#include <cstring>
#include <vector>
#include "pct_device.cuh"

namespace {

struct FileH {
    FILE* f = nullptr;
    ~FileH() {
        if (f) fclose(f);
    }
};

__global__ void k_split_voxel(DevGeom g, int64_t n, const uint32_t* __restrict__ first, int* __restrict__ vx,
                              int* __restrict__ vy, int* __restrict__ vz) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t v = first[i];
    uint32_t C = (uint32_t)g.columns, R = (uint32_t)g.rows;
    vx[i] = (int)(v % C);
    vy[i] = (int)((v / C) % R);
    vz[i] = (int)(v / (C * R));
}

__global__ void k_join_voxel(DevGeom g, int64_t n, const int* __restrict__ vx, const int* __restrict__ vy,
                             const int* __restrict__ vz, uint32_t* __restrict__ first) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    first[i] = (uint32_t)(vx[i] + g.columns * vy[i] + g.rows * g.columns * vz[i]);
}

/* rows of the reference files (linear order) into the row slots (stored order) */
__global__ void k_rows_to_slots(DevGeom g, int64_t total, const uint32_t* __restrict__ src,
                                uint32_t* __restrict__ dst) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < total) dst[k] = dev_to_brick(g, src[k]);
}

__global__ void k_len_from_off(int64_t n, const int64_t* __restrict__ off, int* __restrict__ len) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) len[i] = (int)(off[i + 1] - off[i]);
}

}  // namespace

/* k_row_norms lives with the MLP kernels */
pct_status pct_stage_row_norms(pct_ctx* c);

extern "C" pct_status pct_write_mlp_endpoints(pct_ctx* c, const char* path) {
    if (!c || !path) return pct_fail(PCT_ERR_ARGUMENT, "pct_write_mlp_endpoints: null argument");
    PCT_TRY(c->set_device());
    if (c->stage < ST_ENDPOINTS) return pct_fail(PCT_ERR_STATE, "pct_write_mlp_endpoints needs the MLP endpoints");
    const int64_t n = c->h.n;
    if (n > 0xffffffffLL) return pct_fail(PCT_ERR_OVERFLOW, "pct_write_mlp_endpoints: %lld histories", (long long)n);
    std::vector<int> vxyz((size_t)3 * (size_t)(n > 0 ? n : 1));
    std::vector<float> f((size_t)11 * (size_t)(n > 0 ? n : 1));
    std::vector<int> bin((size_t)(n > 0 ? n : 1));
    if (n > 0) {
        DevBuf tmp;
        PCT_TRY(tmp.alloc(sizeof(int) * 3 * (size_t)n));
        int* d = tmp.as<int>();
        k_split_voxel<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, c->h.first_voxel.as<uint32_t>(), d, d + n,
                                                                    d + 2 * n);
        ++c->launches;
        PCT_CUDA(cudaMemcpyAsync(vxyz.data(), d, sizeof(int) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
        PCT_CUDA(cudaMemcpyAsync(bin.data(), c->h.bin_num.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
        DevBuf* src[11] = {&c->h.wepl, &c->h.x_entry, &c->h.y_entry, &c->h.z_entry, &c->h.x_exit, &c->h.y_exit,
                           &c->h.z_exit, &c->h.xy_entry_angle, &c->h.xz_entry_angle, &c->h.xy_exit_angle,
                           &c->h.xz_exit_angle};
        for (int k = 0; k < 11; ++k)
            PCT_CUDA(cudaMemcpyAsync(f.data() + (size_t)k * n, src[k]->p, sizeof(float) * n, cudaMemcpyDeviceToHost,
                                     c->stream));
        PCT_CUDA(cudaStreamSynchronize(c->stream));
        tmp.release();
    }
    FileH fh;
    fh.f = fopen(path, "wb");
    if (!fh.f) return pct_fail(PCT_ERR_IO, "%s: cannot create", path);
    const uint32_t N = (uint32_t)n;
    bool ok = fwrite(&N, 4, 1, fh.f) == 1;
    ok = ok && (n == 0 || fwrite(vxyz.data(), sizeof(int), 3 * (size_t)n, fh.f) == 3 * (size_t)n);
    ok = ok && (n == 0 || fwrite(bin.data(), sizeof(int), (size_t)n, fh.f) == (size_t)n);
    ok = ok && (n == 0 || fwrite(f.data(), sizeof(float), 11 * (size_t)n, fh.f) == 11 * (size_t)n);
    if (!ok) return pct_fail(PCT_ERR_IO, "%s: write failed", path);
    return PCT_OK;
}

extern "C" pct_status pct_read_mlp_endpoints(pct_ctx* c, const char* path) {
    if (!c || !path) return pct_fail(PCT_ERR_ARGUMENT, "pct_read_mlp_endpoints: null argument");
    PCT_TRY(c->set_device());
    FileH fh;
    fh.f = fopen(path, "rb");
    if (!fh.f) return pct_fail(PCT_ERR_IO, "%s: cannot open", path);
    fseek(fh.f, 0, SEEK_END);
    const long size = ftell(fh.f);
    rewind(fh.f);
    uint32_t N = 0;
    if (fread(&N, 4, 1, fh.f) != 1) return pct_fail(PCT_ERR_IO, "%s: truncated", path);
    const int64_t n = N;
    if (4 + 60 * n != size) return pct_fail(PCT_ERR_IO, "%s: %ld bytes, expected %lld for %u histories", path, size,
                                            (long long)(4 + 60 * n), N);
    std::vector<int> vxyz((size_t)3 * (size_t)(n > 0 ? n : 1)), bin((size_t)(n > 0 ? n : 1));
    std::vector<float> f((size_t)11 * (size_t)(n > 0 ? n : 1));
    if (n > 0 && (fread(vxyz.data(), sizeof(int), 3 * (size_t)n, fh.f) != 3 * (size_t)n ||
                  fread(bin.data(), sizeof(int), (size_t)n, fh.f) != (size_t)n ||
                  fread(f.data(), sizeof(float), 11 * (size_t)n, fh.f) != 11 * (size_t)n))
        return pct_fail(PCT_ERR_IO, "%s: read failed", path);
    PCT_TRY(c->h.reserve(n > 0 ? n : 1, c->stream));
    c->h.n = n;
    if (n > 0) {
        DevBuf tmp;
        PCT_TRY(tmp.alloc(sizeof(int) * 3 * (size_t)n));
        int* d = tmp.as<int>();
        PCT_CUDA(cudaMemcpyAsync(d, vxyz.data(), sizeof(int) * 3 * n, cudaMemcpyHostToDevice, c->stream));
        k_join_voxel<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(c->dg, n, d, d + n, d + 2 * n,
                                                                   c->h.first_voxel.as<uint32_t>());
        ++c->launches;
        PCT_CUDA(cudaMemcpyAsync(c->h.bin_num.p, bin.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
        DevBuf* dst[11] = {&c->h.wepl, &c->h.x_entry, &c->h.y_entry, &c->h.z_entry, &c->h.x_exit, &c->h.y_exit,
                           &c->h.z_exit, &c->h.xy_entry_angle, &c->h.xz_entry_angle, &c->h.xy_exit_angle,
                           &c->h.xz_exit_angle};
        for (int k = 0; k < 11; ++k)
            PCT_CUDA(cudaMemcpyAsync(dst[k]->p, f.data() + (size_t)k * n, sizeof(float) * n, cudaMemcpyHostToDevice,
                                     c->stream));
        PCT_CUDA(cudaMemsetAsync(c->h.bin_valid.p, 1, (size_t)n, c->stream));
        PCT_CUDA(cudaMemsetAsync(c->h.failed.p, 0, (size_t)n, c->stream));
        PCT_CUDA(cudaStreamSynchronize(c->stream));
        tmp.release();
    }
    /* an iterate to start from: the context's x0, else zeros (PCT_ZEROS) until pct_set_image */
    const size_t vb = sizeof(float) * (size_t)c->geo.num_voxels;
    if (!c->x0.p || !c->x.p) {
        PCT_TRY(c->x0.alloc(vb));
        PCT_TRY(c->x.alloc(vb));
        PCT_CUDA(cudaMemsetAsync(c->x0.p, 0, vb, c->stream));
        PCT_CUDA(cudaMemsetAsync(c->x.p, 0, vb, c->stream));
    }
    c->counts.reconstruction_histories = n;
    c->stage = ST_ENDPOINTS;
    c->diag_ready = 0;
    pct_drop_release_graph(c);
    return PCT_OK;
}

extern "C" pct_status pct_write_mlp_paths(pct_ctx* c, const char* path) {
    if (!c || !path) return pct_fail(PCT_ERR_ARGUMENT, "pct_write_mlp_paths: null argument");
    PCT_TRY(c->set_device());
    if (c->stage < ST_ROWS) return pct_fail(PCT_ERR_STATE, "pct_write_mlp_paths needs the MLP rows");
    const int64_t n = c->h.n;
    int64_t total = 0;
    PCT_TRY(pct_rows_dense(c, &total, &c->dense_off, &c->dense_rows));
    std::vector<int64_t> off((size_t)n + 1);
    std::vector<uint32_t> rows((size_t)(total > 0 ? total : 1));
    PCT_CUDA(cudaMemcpyAsync(off.data(), c->dense_off.p, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    if (total > 0)
        PCT_CUDA(cudaMemcpyAsync(rows.data(), c->dense_rows.p, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost,
                                 c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    FileH fh;
    fh.f = fopen(path, "wb");
    if (!fh.f) return pct_fail(PCT_ERR_IO, "%s: cannot create", path);
    bool ok = fprintf(fh.f, "%u\n", (unsigned)n) > 0;
    for (int64_t i = 0; ok && i < n; ++i) {
        const uint32_t cnt = (uint32_t)(off[i + 1] - off[i]);
        ok = fwrite(&cnt, 4, 1, fh.f) == 1 && (cnt == 0 || fwrite(rows.data() + off[i], 4, cnt, fh.f) == cnt);
    }
    if (!ok) return pct_fail(PCT_ERR_IO, "%s: write failed", path);
    return PCT_OK;
}

extern "C" pct_status pct_read_mlp_paths(pct_ctx* c, const char* path) {
    if (!c || !path) return pct_fail(PCT_ERR_ARGUMENT, "pct_read_mlp_paths: null argument");
    PCT_TRY(c->set_device());
    if (c->stage < ST_ENDPOINTS) return pct_fail(PCT_ERR_STATE, "pct_read_mlp_paths needs the MLP endpoints");
    FileH fh;
    fh.f = fopen(path, "rb");
    if (!fh.f) return pct_fail(PCT_ERR_IO, "%s: cannot open", path);
    /* "<N>\n" */
    char line[32];
    int k = 0, ch;
    while (k < 31 && (ch = fgetc(fh.f)) != EOF && ch != '\n') line[k++] = (char)ch;
    line[k] = 0;
    if (ch != '\n' || k == 0) return pct_fail(PCT_ERR_IO, "%s: bad header", path);
    char* endp = nullptr;
    unsigned long long N = strtoull(line, &endp, 10);
    if (!endp || *endp != 0) return pct_fail(PCT_ERR_IO, "%s: bad header", path);
    const int64_t n = c->h.n;
    if ((int64_t)N != n)
        return pct_fail(PCT_ERR_ARGUMENT, "%s: %llu paths for %lld histories", path, N, (long long)n);
    std::vector<int64_t> off((size_t)n + 1, 0);
    std::vector<uint32_t> rows;
    for (int64_t i = 0; i < n; ++i) {
        uint32_t cnt = 0;
        if (fread(&cnt, 4, 1, fh.f) != 1) return pct_fail(PCT_ERR_IO, "%s: truncated at path %lld", path, (long long)i);
        if (cnt > (1u << 20)) return pct_fail(PCT_ERR_IO, "%s: path %lld has %u entries", path, (long long)i, cnt);
        size_t at = rows.size();
        rows.resize(at + cnt);
        if (cnt && fread(rows.data() + at, 4, cnt, fh.f) != cnt)
            return pct_fail(PCT_ERR_IO, "%s: truncated at path %lld", path, (long long)i);
        off[i + 1] = off[i] + cnt;
    }
    const int64_t total = off[n];
    PCT_TRY(c->row_offsets.alloc(sizeof(int64_t) * (n + 1)));
    PCT_TRY(c->row_len.alloc(sizeof(int) * (n > 0 ? n : 1)));
    PCT_TRY(c->rows.alloc(sizeof(uint32_t) * (total > 0 ? total : 1)));
    PCT_TRY(c->chord.alloc(sizeof(float) * (n > 0 ? n : 1)));
    PCT_TRY(c->row_scale.alloc(sizeof(float) * (n > 0 ? n : 1)));
    PCT_CUDA(cudaMemcpyAsync(c->row_offsets.p, off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, c->stream));
    if (total > 0) {
        DevBuf tmp;
        PCT_TRY(tmp.alloc(sizeof(uint32_t) * total));
        PCT_CUDA(cudaMemcpyAsync(tmp.p, rows.data(), sizeof(uint32_t) * total, cudaMemcpyHostToDevice, c->stream));
        k_rows_to_slots<<<pct_grid_for(total, 256), 256, 0, c->stream>>>(c->dg, total, tmp.as<uint32_t>(),
                                                                        c->rows.as<uint32_t>());
        ++c->launches;
        PCT_CUDA(cudaStreamSynchronize(c->stream));
        tmp.release();
    }
    if (n > 0) {
        k_len_from_off<<<pct_grid_for(n, 256), 256, 0, c->stream>>>(n, c->row_offsets.as<int64_t>(), c->row_len.as<int>());
        ++c->launches;
    }
    c->row_capacity = total;
    PCT_TRY(pct_stage_row_norms(c));
    c->counts.row_entries = -1;
    c->diag_ready = 0;
    pct_drop_release_graph(c);
    c->stage = ST_ROWS;
    return PCT_OK;
}

extern "C" pct_status pct_write_image(pct_ctx* c, pct_array which, const char* path) {
    if (!c || !path) return pct_fail(PCT_ERR_ARGUMENT, "pct_write_image: null argument");
    if (which != PCT_ARR_X && which != PCT_ARR_X0 && which != PCT_ARR_FBP_IMAGE)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_write_image: not a float image");
    std::vector<float> img((size_t)c->geo.num_voxels);
    size_t bytes = img.size() * sizeof(float);
    PCT_TRY(pct_get_array(c, which, img.data(), &bytes));
    FileH fh;
    fh.f = fopen(path, "wb");
    if (!fh.f) return pct_fail(PCT_ERR_IO, "%s: cannot create", path);
    if (fwrite(img.data(), 1, bytes, fh.f) != bytes) return pct_fail(PCT_ERR_IO, "%s: write failed", path);
    return PCT_OK;
}

extern "C" pct_status pct_read_image(pct_ctx* c, const char* path) {
    if (!c || !path) return pct_fail(PCT_ERR_ARGUMENT, "pct_read_image: null argument");
    std::vector<float> img((size_t)c->geo.num_voxels);
    FileH fh;
    fh.f = fopen(path, "rb");
    if (!fh.f) return pct_fail(PCT_ERR_IO, "%s: cannot open", path);
    if (fread(img.data(), sizeof(float), img.size(), fh.f) != img.size() || fgetc(fh.f) != EOF)
        return pct_fail(PCT_ERR_IO, "%s: not an image of %d voxels", path, c->geo.num_voxels);
    return pct_set_image(c, img.data());
}
