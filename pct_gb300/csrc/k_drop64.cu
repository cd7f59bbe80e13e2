/*
 * Binary64 DROP (pct_drop_fp64): the block iteration of the binary32 scatter
 * form (k_drop.cu) with every quantity in binary64, the way the reference's
 * host DROP keeps its update accumulator (DROP_blocks / DROP_update,
 * .cu:8023-8055) and the oracle its image: the row's chord
 * (EffectiveChordLength_GPU, .cu:4974-4995, unrounded), the dot c sum x, the
 * norm ||a_i||^2 = c^2 n, the update c lambda (b - c sum x) / ||a_i||^2 added
 * with binary64 atomics, and the relaxation x += x_update / s_j
 * (image_update_GPU, .cu:5900-5938).
 *
 * It states the error of the binary32 path against a binary64 run of the same
 * iterations on the same rows at full size.  It is a validation path (bound by
 * binary64 L2 reductions), not a fast path.
 */
#include <cstring>
#include "pct_device.cuh"


int pct_drop_num_blocks(const pct_ctx* c);                                  /* k_drop.cu */
void pct_drop_block_range(const pct_ctx* c, int k, int64_t* s, int64_t* e); /* k_drop.cu */
pct_status pct_row_chords64(pct_ctx* c, double* out);                       /* k_mlp.cu */

namespace {

constexpr int D64_THREADS = 256;
constexpr int D64_WARPS = D64_THREADS / 32;

/* One warp per row (grid-stride): the reference's row update in binary64, in
 * the operation order of DROP_blocks (.cu:8023-8043). */
__global__ void __launch_bounds__(D64_THREADS) k_drop_rows64(int64_t start, int64_t end,
                                                             const int64_t* __restrict__ row_start,
                                                             const int* __restrict__ row_len,
                                                             const uint32_t* __restrict__ rows,
                                                             const double* __restrict__ chord,
                                                             const float* __restrict__ wepl, double lambda,
                                                             const double* __restrict__ x, double* __restrict__ upd,
                                                             uint32_t nv, double* __restrict__ resid) {
    __shared__ double sres[D64_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double r2 = 0.0;
    for (int64_t i = start + (int64_t)blockIdx.x * D64_WARPS + w; i < end; i += (int64_t)gridDim.x * D64_WARPS) {
        const int64_t a = row_start[i];
        const int len = row_len[i];
        double dot = 0.0;
        for (int q = lane; q < len; q += 32) {
            const uint32_t v = rows[a + q];
            if (v < nv) dot += x[v];
        }
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        const double c = chord[i];
        dot *= c;
        const double aa = (c * c) * (double)len;
        const double res = (double)wepl[i] - dot;
        const double value = c * (res / aa) * lambda;
        for (int q = lane; q < len; q += 32) {
            const uint32_t v = rows[a + q];
            if (v < nv) atomicAdd(upd + v, value);
        }
        r2 += res * res;
    }
    if (lane == 0) sres[w] = r2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < D64_WARPS; ++k) s += sres[k];
        if (s != 0.0) atomicAdd(resid, s);
    }
}

/* x += x_update / s_j where s_j > 0; x_update cleared (DROP_update, .cu:8044-8055) */
__global__ void k_drop_relax64(int nv, const uint32_t* __restrict__ cnt, double* __restrict__ x,
                               double* __restrict__ upd) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const uint32_t s = cnt[v];
    if (s > 0) {
        x[v] += upd[v] / s;
        upd[v] = 0.0;
    }
}

__global__ void k_to_brick64(DevGeom g, const double* __restrict__ lin, double* __restrict__ brk) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < g.num_voxels) brk[dev_to_brick(g, (uint32_t)v)] = lin[v];
}
__global__ void k_from_brick64(DevGeom g, const double* __restrict__ brk, double* __restrict__ lin) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < g.num_voxels) lin[v] = brk[dev_to_brick(g, (uint32_t)v)];
}

__global__ void k_sum_sq64(int64_t n, const float* __restrict__ wepl, double* __restrict__ out) {
    __shared__ double red[8];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double b = wepl[i];
        s += b * b;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        atomicAdd(out, t);
    }
}

}  // namespace

extern "C" pct_status pct_drop_fp64(pct_ctx* c, int iterations, double* x, pct_drop_stats* stats) {
    if (!c || !x) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_fp64: null argument");
    PCT_TRY(c->set_device());
    if (c->stage != ST_ROWS) return pct_fail(PCT_ERR_STATE, "pct_drop_fp64 needs MLP rows");
    if (iterations < 0 || iterations > 64) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_fp64: %d iterations", iterations);
    if (c->cfg.drop_variant != PCT_DROP_STANDARD)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_fp64: only the standard DROP update");
    if (c->allreduce || c->num_shards != 1) return pct_fail(PCT_ERR_STATE, "pct_drop_fp64: not for a shard");
    PCT_TRY(pct_drop_prepare(c));
    if (c->drop_mode == PCT_DROP_TILED)
        return pct_fail(PCT_ERR_STATE, "pct_drop_fp64 needs the scatter or sorted form's diagonal counts");
    const int nv = c->geo.num_voxels;
    const int64_t n = c->h.n;
    const size_t vb = sizeof(double) * (size_t)nv;
    PCT_TRY(c->d64_x.alloc(vb));
    PCT_TRY(c->d64_upd.alloc(vb));
    PCT_TRY(c->d64_chord.alloc(sizeof(double) * (size_t)(n > 0 ? n : 1)));
    PCT_TRY(c->d64_res.alloc(sizeof(double) * 66));
    double* dx = c->d64_x.as<double>();
    double* du = c->d64_upd.as<double>();
    double* dres = c->d64_res.as<double>(); /* [0, 64): per iteration, 64: ||b||^2 */
    PCT_TRY(pct_row_chords64(c, c->d64_chord.as<double>()));
    PCT_CUDA(cudaMemsetAsync(dres, 0, sizeof(double) * 66, c->stream));
    if (n > 0) k_sum_sq64<<<304, 256, 0, c->stream>>>(n, c->h.wepl.as<float>(), dres + 64);
    /* the caller's image (linear order) into the rows' voxel order; du is the staging */
    PCT_CUDA(cudaMemcpyAsync(du, x, vb, cudaMemcpyHostToDevice, c->stream));
    k_to_brick64<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(c->dg, du, dx);
    PCT_CUDA(cudaMemsetAsync(du, 0, vb, c->stream));
    c->launches += 2;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || sms < 1) sms = 1;
    cudaEvent_t e0, e1;
    PCT_CUDA(cudaEventCreate(&e0));
    PCT_CUDA(cudaEventCreate(&e1));
    PCT_CUDA(cudaEventRecord(e0, c->stream));
    const int nb = c->num_blocks;
    for (int it = 0; it < iterations; ++it) {
        for (int k = 0; k < nb; ++k) {
            int64_t s, e;
            pct_drop_block_range(c, k, &s, &e);
            if (e == s) continue;
            const int64_t need = (e - s + D64_WARPS - 1) / D64_WARPS;
            const unsigned grid = (unsigned)(need < (int64_t)sms * 8 ? need : (int64_t)sms * 8);
            k_drop_rows64<<<grid, D64_THREADS, 0, c->stream>>>(
                s, e, c->row_offsets.as<int64_t>(), c->row_len.as<int>(), c->rows.as<uint32_t>(),
                c->d64_chord.as<double>(), c->h.wepl.as<float>(), (double)c->cfg.lambda, dx, du, (uint32_t)nv,
                dres + it);
            k_drop_relax64<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(
                nv, c->block_diag.as<uint32_t>() + (size_t)k * nv, dx, du);
            c->launches += 2;
        }
    }
    PCT_CUDA(cudaEventRecord(e1, c->stream));
    k_from_brick64<<<pct_grid_for(nv, 256), 256, 0, c->stream>>>(c->dg, dx, du);
    ++c->launches;
    PCT_CUDA(cudaGetLastError());
    PCT_CUDA(cudaMemcpyAsync(x, du, vb, cudaMemcpyDeviceToHost, c->stream));
    double res[66];
    PCT_CUDA(cudaMemcpyAsync(res, dres, sizeof(res), cudaMemcpyDeviceToHost, c->stream));
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->iterations_run = iterations;
        for (int k = 0; k < iterations; ++k) stats->residual[k] = res[64] > 0 ? sqrt(res[k] / res[64]) : 0.0;
        stats->seconds = ms * 1e-3;
        stats->drop_form = c->drop_mode;
    }
    return PCT_OK;
}
