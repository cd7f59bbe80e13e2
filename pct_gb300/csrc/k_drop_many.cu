/*
 * DROP iterations of many scans in one persistent launch per iteration.
 *
 * The reference reconstructs one scan per run: its block loop
 * (src/pCT_Reconstruction_Data_Segments.cu:6795-6844) launches the block
 * update and the image update of each block in turn.  Here every scan, each
 * with its own block size, advances at most one block per level inside one
 * cooperative launch:
 *
 *   level L, rows    the rows of the blocks placed at level L (one block of
 *                    each of several scans), laid end to end, split over all
 *                    warps of the launch the way the scatter form splits one
 *                    block (warp w takes rows w, w + W, ...): the dot with the
 *                    iterate, the binary32 update value, one L2 reduction per
 *                    row entry, the binary64 squared residual;
 *   grid barrier
 *   level L, relax   x += x_update / s_j and x_update = 0 over the voxels of
 *                    the same scans, split over all threads;
 *   grid barrier, level L + 1.
 *
 * There are as many levels as the longest chain of blocks, and each scan's
 * blocks are spread evenly over them, so that scans of uneven history counts
 * and block sizes share every level's launch width and no scan runs on alone
 * with the device mostly idle.  The barriers are counters in global
 * memory (all CTAs are resident: the launch is cooperative); each wait is
 * bounded: after BAR_SPIN polls a CTA raises the abort flag, every CTA
 * leaves, and the host reports an error.  Iterates and updates written
 * during the launch are read with L2-only loads (ld.global.cg) after the
 * barrier's acquire fence.  One CUDA graph holds an iteration: the reset of
 * the barrier, the launch and the per-scan residual slots.
 */
#include <cstring>
#include <utility>
#include <vector>
#include "pct_device.cuh"

namespace {

constexpr int MANY_THREADS = 256;
constexpr int MANY_WARPS = MANY_THREADS / 32;
constexpr int MANY_REG = 8;               /* row entries per lane held in registers */
constexpr long long BAR_SPIN = 1ll << 20; /* polls of a grid barrier (sleeps of up to BAR_NAP_MAX ns) */
constexpr unsigned BAR_NAP_MAX = 1024;
constexpr int MANY_MAX_SCANS = 256;       /* residual accumulators per CTA (shared memory) */

struct ManyScan {
    const int64_t* row_start;
    const int* row_len;
    const uint32_t* rows;
    const float* chord;
    const float* row_scale;
    const float* wepl;
    float* x;             /* the iterate in the rows' voxel order */
    float* upd;
    const uint32_t* diag; /* s_j of every block, num_blocks x nv */
    double* resid;        /* squared-residual accumulator of the iteration */
    int64_t n, block_size;
    uint32_t nv;
    int num_blocks;
    float lambda;
    int vec4;             /* nv % 4 == 0: 16-byte relax */
};

/* One scan's share of a level: its block `block`, rows [row0, row0 + rows) laid
 * from `row_at` in the level's row space, its relax items (voxels, or groups
 * of four) from `item_at` in the level's item space. */
struct ManySeg {
    int scan, block;
    int64_t row0, rows, row_at;
    int64_t items, item_at;
};

struct ManyLevel {
    int seg0, nseg;
    int64_t rows, items;
};

/* ctl[0]: barrier arrivals, ctl[1]: abort flag, ctl[2]: barrier that ran out */

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) { return *(const volatile unsigned*)p; }

/* Grid barrier number k (1, 2, ...): false when a wait ran out or the launch aborted. */
__device__ bool many_barrier(unsigned* ctl, unsigned k) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence(); /* release: this CTA's writes before its arrival */
        atomicAdd(ctl, 1u);
        const unsigned target = k * gridDim.x;
        ok = 0;
        /* polls back off to one per few microseconds: hundreds of CTAs polling one
         * address would load its L2 slice while the other CTAs still work */
        unsigned nap = 256;
        for (long long s = 0; s < BAR_SPIN; ++s) {
            if (ld_volatile(ctl) >= target) {
                ok = 1;
                break;
            }
            if (ld_volatile(ctl + 1)) break;
            __nanosleep(nap);
            if (nap < BAR_NAP_MAX) nap <<= 1;
        }
        if (!ok && !ld_volatile(ctl + 1)) {
            atomicExch(ctl + 2, k);
            atomicExch(ctl + 1, 1u);
        }
        __threadfence(); /* acquire: the other CTAs' writes before this CTA's reads */
    }
    __syncthreads();
    return ok != 0;
}

/* A reduction into global memory (red.global.add.f32, no value returned).  The
 * scan table's pointers are generic: an atomicAdd through them compiles to a
 * returning generic atomic, which costs a round trip per row entry. */
__device__ __forceinline__ void red_add(float* p, float v) {
    asm volatile("{\n\t.reg .u64 ga;\n\tcvta.to.global.u64 ga, %0;\n\tred.global.add.f32 [ga], %1;\n\t}"
                 :: "l"(p), "f"(v) : "memory");
}

/* Row i of scan S; its squared residual goes to (r2, pend, nrow). */
__device__ __forceinline__ void many_row(const ManyScan& S, int64_t i, double& r2, float& pend, int& nrow) {
    const int lane = threadIdx.x & 31;
    const uint32_t nv = S.nv;
    const uint32_t* __restrict__ rows = S.rows;
    const float* x = S.x;
    float* upd = S.upd;
    const int64_t a = S.row_start[i];
    const int len = S.row_len[i];
    uint32_t e[MANY_REG];
#pragma unroll
    for (int k = 0; k < MANY_REG; ++k) {
        const int q = lane + 32 * k;
        e[k] = q < len ? __ldcs(rows + a + q) : 0xffffffffu;
    }
    float dot = 0.0f;
#pragma unroll
    for (int k = 0; k < MANY_REG; ++k) dot += e[k] < nv ? __ldcg(x + e[k]) : 0.0f;
    for (int q = 32 * MANY_REG + lane; q < len; q += 32) {
        const uint32_t v = __ldcs(rows + a + q);
        if (v < nv) dot += __ldcg(x + v);
    }
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    const float res = fmaf(-S.chord[i], dot, S.wepl[i]);
    const float value = (res * S.row_scale[i]) * S.lambda;
#pragma unroll
    for (int k = 0; k < MANY_REG; ++k)
        if (e[k] < nv) red_add(upd + e[k], value);
    for (int q = 32 * MANY_REG + lane; q < len; q += 32) {
        const uint32_t v = __ldcs(rows + a + q);
        if (v < nv) red_add(upd + v, value);
    }
    if (lane == (nrow & 31)) pend = res;
    if ((++nrow & 31) == 0) {
        r2 = fma((double)pend, (double)pend, r2);
        pend = 0.0f;
    }
}

/* The warp's pending squared residuals into the CTA's accumulator of `scan`. */
__device__ __forceinline__ void flush_resid(double* sres, int scan, double& r2, float& pend) {
    r2 = fma((double)pend, (double)pend, r2);
    pend = 0.0f;
    for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    if ((threadIdx.x & 31) == 0 && r2 != 0.0) atomicAdd(sres + scan, r2);
    r2 = 0.0;
}

__global__ void __launch_bounds__(MANY_THREADS) k_drop_many(const ManyScan* __restrict__ scans, int nscans,
                                                            const ManyLevel* __restrict__ levels, int nlevels,
                                                            const ManySeg* __restrict__ segs,
                                                            unsigned* __restrict__ ctl) {
    __shared__ double sres[MANY_MAX_SCANS];
    for (int s = threadIdx.x; s < nscans; s += MANY_THREADS) sres[s] = 0.0;
    __syncthreads();
    const int64_t nwarps = (int64_t)gridDim.x * MANY_WARPS;
    const int64_t gwarp = (int64_t)blockIdx.x * MANY_WARPS + (threadIdx.x >> 5);
    const int64_t nthreads = (int64_t)gridDim.x * MANY_THREADS;
    const int64_t gthread = (int64_t)blockIdx.x * MANY_THREADS + threadIdx.x;
    double r2 = 0.0;
    float pend = 0.0f;
    int nrow = 0;
    unsigned bar = 0;
    for (int L = 0; L < nlevels; ++L) {
        const ManyLevel lv = levels[L];
        /* rows: warp-strided over the level's row space, segment by segment */
        int sg = lv.seg0, rscan = -1;
        for (int64_t g = gwarp; g < lv.rows; g += nwarps) {
            while (g >= segs[sg].row_at + segs[sg].rows) ++sg;
            const int scan = segs[sg].scan;
            if (scan != rscan) {
                if (rscan >= 0) flush_resid(sres, rscan, r2, pend);
                rscan = scan;
            }
            many_row(scans[scan], segs[sg].row0 + (g - segs[sg].row_at), r2, pend, nrow);
        }
        if (rscan >= 0) flush_resid(sres, rscan, r2, pend);
        if (!many_barrier(ctl, ++bar)) return;
        /* relax: thread-strided over the level's item space */
        sg = lv.seg0;
        for (int64_t g = gthread; g < lv.items; g += nthreads) {
            while (g >= segs[sg].item_at + segs[sg].items) ++sg;
            const ManyScan& S = scans[segs[sg].scan];
            const int64_t q = g - segs[sg].item_at;
            const uint32_t* cnt = S.diag + (size_t)segs[sg].block * S.nv;
            if (S.vec4) {
                const uint4 s4 = __ldg(reinterpret_cast<const uint4*>(cnt) + q);
                if ((s4.x | s4.y | s4.z | s4.w) == 0u) continue;
                float4* xp = reinterpret_cast<float4*>(S.x) + q;
                float4* up = reinterpret_cast<float4*>(S.upd) + q;
                const float4 u = __ldcg(up);
                float4 xv = __ldcg(xp);
                if (s4.x > 0) xv.x += u.x / (float)s4.x;
                if (s4.y > 0) xv.y += u.y / (float)s4.y;
                if (s4.z > 0) xv.z += u.z / (float)s4.z;
                if (s4.w > 0) xv.w += u.w / (float)s4.w;
                __stcg(xp, xv);
                __stcg(up, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
            } else {
                const uint32_t s1 = __ldg(cnt + q);
                if (s1 == 0u) continue;
                __stcg(S.x + q, __ldcg(S.x + q) + __ldcg(S.upd + q) / (float)s1);
                __stcg(S.upd + q, 0.0f);
            }
        }
        if (!many_barrier(ctl, ++bar)) return;
    }
    __syncthreads();
    for (int s = threadIdx.x; s < nscans; s += MANY_THREADS)
        if (sres[s] != 0.0) atomicAdd(scans[s].resid, sres[s]);
}

/* Per scan: the iteration's squared residual into slot `it`, accumulator cleared. */
__global__ void k_many_store_resid(int count, double* const* __restrict__ acc, int it) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count) return;
    double* a = acc[s];
    a[it] = a[PCT_DROP_MAXIT];
    a[PCT_DROP_MAXIT] = 0.0;
}

struct DevMem {
    void* p = nullptr;
    ~DevMem() {
        if (p) cudaFree(p);
    }
};

}  // namespace

extern "C" pct_status pct_drop_many(pct_ctx* const* ctxs, int count, int iterations, pct_drop_stats* stats) {
    if (!ctxs || count < 1 || iterations < 0) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: bad arguments");
    if (count > MANY_MAX_SCANS) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: at most %d scans", MANY_MAX_SCANS);
    if (iterations > PCT_DROP_MAXIT)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: at most %d iterations per call", PCT_DROP_MAXIT);
    pct_ctx* c0 = ctxs[0];
    for (int s = 0; s < count; ++s) {
        pct_ctx* c = ctxs[s];
        if (!c) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: null context %d", s);
        if (c->device != c0->device) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: contexts on different devices");
        for (int t = 0; t < s; ++t)
            if (ctxs[t] == c) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: context %d given twice", s);
        if (c->stage != ST_ROWS) return pct_fail(PCT_ERR_STATE, "pct_drop_many: context %d has no MLP rows", s);
        if (c->cfg.drop_form != PCT_DROP_SCATTER || c->cfg.drop_variant != PCT_DROP_STANDARD || c->allreduce ||
            c->num_shards != 1)
            return pct_fail(PCT_ERR_ARGUMENT,
                            "pct_drop_many: context %d: the standard update in the scatter form, unsharded", s);
    }
    PCT_TRY(c0->set_device());
    /* per scan: block structures, zero update, iterate in the rows' voxel order, residual slots */
    for (int s = 0; s < count; ++s) {
        PCT_TRY(pct_drop_begin(ctxs[s]));
        PCT_CUDA(cudaStreamSynchronize(ctxs[s]->stream));
    }
    std::vector<ManyScan> hs(count);
    std::vector<double*> hres(count);
    int nlevels = 0;
    for (int s = 0; s < count; ++s) {
        pct_ctx* c = ctxs[s];
        ManyScan& S = hs[s];
        S.row_start = c->row_offsets.as<int64_t>();
        S.row_len = c->row_len.as<int>();
        S.rows = c->rows.as<uint32_t>();
        S.chord = c->chord.as<float>();
        S.row_scale = c->row_scale.as<float>();
        S.wepl = c->h.wepl.as<float>();
        S.x = c->dg.brick ? c->x_brick.as<float>() : c->x.as<float>();
        S.upd = c->x_update.as<float>();
        S.diag = c->block_diag.as<uint32_t>();
        S.resid = c->drop_resid.as<double>() + PCT_DROP_MAXIT;
        S.n = c->h.n;
        S.block_size = c->cfg.block_size;
        S.nv = (uint32_t)c->geo.num_voxels;
        S.num_blocks = c->num_blocks;
        S.lambda = c->cfg.lambda;
        S.vec4 = S.nv % 4 == 0;
        hres[s] = c->drop_resid.as<double>();
        if ((int64_t)S.num_blocks * S.block_size < S.n)
            return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: context %d: block layout", s);
        nlevels = S.num_blocks > nlevels ? S.num_blocks : nlevels;
    }
    /* Scan s, with nb_s blocks, does its block b at level floor(b * levels / nb_s):
     * its blocks stay in order, one per level at most, spread evenly over the
     * launch.  Within a level the scans' rows and relax items are laid end to end. */
    std::vector<std::vector<std::pair<int, int>>> at((size_t)nlevels);
    for (int s = 0; s < count; ++s)
        for (int b = 0; b < hs[s].num_blocks; ++b)
            at[(size_t)((int64_t)b * nlevels / hs[s].num_blocks)].push_back({s, b});
    std::vector<ManyLevel> levels;
    std::vector<ManySeg> segs;
    for (int L = 0; L < nlevels; ++L) {
        ManyLevel lv{(int)segs.size(), 0, 0, 0};
        for (const auto& sb : at[(size_t)L]) {
            const int s = sb.first, b = sb.second;
            const ManyScan& S = hs[s];
            const int64_t r0 = (int64_t)b * S.block_size;
            const int64_t rn = (r0 + S.block_size < S.n ? r0 + S.block_size : S.n) - r0;
            const int64_t items = S.vec4 ? (int64_t)S.nv / 4 : (int64_t)S.nv;
            segs.push_back({s, b, r0, rn, lv.rows, items, lv.items});
            lv.rows += rn;
            lv.items += items;
            ++lv.nseg;
        }
        levels.push_back(lv);
    }
    int sms = 0, per_sm = 0;
    PCT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c0->device));
    PCT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_drop_many, MANY_THREADS, 0));
    if (per_sm < 1) return pct_fail(PCT_ERR_CUDA, "pct_drop_many: kernel does not fit on an SM");
    const unsigned grid = (unsigned)(sms * per_sm);
    if ((int64_t)2 * nlevels * grid > 0xffffffffll) return pct_fail(PCT_ERR_ARGUMENT, "pct_drop_many: too many levels");
    DevMem d_scans, d_levels, d_segs, d_ctl, d_res;
    PCT_CUDA(cudaMalloc(&d_scans.p, sizeof(ManyScan) * count));
    PCT_CUDA(cudaMalloc(&d_levels.p, sizeof(ManyLevel) * (nlevels > 0 ? nlevels : 1)));
    PCT_CUDA(cudaMalloc(&d_segs.p, sizeof(ManySeg) * (segs.empty() ? 1 : segs.size())));
    PCT_CUDA(cudaMalloc(&d_ctl.p, sizeof(unsigned) * 4));
    PCT_CUDA(cudaMalloc(&d_res.p, sizeof(double*) * count));
    cudaStream_t st = c0->stream;
    PCT_CUDA(cudaMemcpyAsync(d_scans.p, hs.data(), sizeof(ManyScan) * count, cudaMemcpyHostToDevice, st));
    if (nlevels) {
        PCT_CUDA(cudaMemcpyAsync(d_levels.p, levels.data(), sizeof(ManyLevel) * nlevels, cudaMemcpyHostToDevice, st));
        PCT_CUDA(cudaMemcpyAsync(d_segs.p, segs.data(), sizeof(ManySeg) * segs.size(), cudaMemcpyHostToDevice, st));
    }
    PCT_CUDA(cudaMemcpyAsync(d_res.p, hres.data(), sizeof(double*) * count, cudaMemcpyHostToDevice, st));
    const ManyScan* a_scans = (const ManyScan*)d_scans.p;
    const ManyLevel* a_levels = (const ManyLevel*)d_levels.p;
    const ManySeg* a_segs = (const ManySeg*)d_segs.p;
    unsigned* a_ctl = (unsigned*)d_ctl.p;
    double* const* a_res = (double* const*)d_res.p;
    /* one iteration: barrier reset, the cooperative launch (all CTAs resident), the residual slots */
    cudaLaunchConfig_t lc;
    memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3(grid);
    lc.blockDim = dim3(MANY_THREADS);
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    auto enqueue = [&](int it) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(a_ctl, 0, sizeof(unsigned) * 4, st);
        if (e == cudaSuccess && nlevels)
            e = cudaLaunchKernelEx(&lc, k_drop_many, a_scans, count, a_levels, nlevels, a_segs, a_ctl);
        if (e == cudaSuccess) {
            k_many_store_resid<<<(count + 127) / 128, 128, 0, st>>>(count, a_res, it);
            e = cudaGetLastError();
        }
        return e;
    };
    cudaEvent_t e0, e1;
    PCT_CUDA(cudaEventCreate(&e0));
    PCT_CUDA(cudaEventCreate(&e1));
    PCT_CUDA(cudaEventRecord(e0, st));
    std::vector<cudaGraphExec_t> graphs;
    cudaError_t err = cudaSuccess;
    bool use_graphs = true;
    for (int it = 0; it < iterations && err == cudaSuccess; ++it) {
        if (use_graphs) {
            /* one captured graph per iteration (the residual slot differs) */
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (ce == cudaSuccess) {
                const cudaError_t e2 = enqueue(it);
                ce = cudaStreamEndCapture(st, &g);
                if (ce == cudaSuccess) ce = e2;
            }
            if (ce == cudaSuccess) ce = cudaGraphInstantiate(&ge, g, 0);
            if (g) cudaGraphDestroy(g);
            if (ce == cudaSuccess) {
                graphs.push_back(ge);
                err = cudaGraphLaunch(ge, st);
                c0->launches += nlevels ? 2 : 1;
                continue;
            }
            /* a cooperative launch this driver does not capture: launched directly */
            (void)cudaGetLastError();
            use_graphs = false;
        }
        err = enqueue(it);
        c0->launches += nlevels ? 2 : 1;
    }
    PCT_CUDA(cudaEventRecord(e1, st));
    cudaError_t sync = cudaStreamSynchronize(st);
    for (cudaGraphExec_t ge : graphs) cudaGraphExecDestroy(ge);
    if (err != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "pct_drop_many: %s", cudaGetErrorString(err));
    if (sync != cudaSuccess) return pct_fail(PCT_ERR_CUDA, "pct_drop_many: %s", cudaGetErrorString(sync));
    unsigned ctl[4];
    PCT_CUDA(cudaMemcpy(ctl, a_ctl, sizeof(ctl), cudaMemcpyDeviceToHost));
    if (ctl[1]) return pct_fail(PCT_ERR_CUDA, "pct_drop_many: grid barrier %u timed out", ctl[2]);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int s = 0; s < count; ++s) PCT_TRY(pct_drop_end(ctxs[s], iterations, ms, stats ? stats + s : nullptr));
    return PCT_OK;
}
