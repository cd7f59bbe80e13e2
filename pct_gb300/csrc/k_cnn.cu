/*
 * Learned warm start for DROP: a 3D residual CNN on the 5th-generation tensor
 * cores (no reference counterpart; it plugs in where the reference chooses
 * its initial iterate, define_initial_iterate .cu:7191-7224, X_K0 = IMPORT).
 *
 * Network (fixed shape): input = the HYBRID initial iterate x0 = FBP x hull and
 * the hull mask (2 channels, padded to 16); 8 convolutions 3x3x3 with zero
 * padding: 2 -> 32, six 32 -> 32 (ReLU after each of the first seven), 32 -> 1;
 * output = x0 + last convolution (a residual correction of the FBP start).
 * Weights and activations bf16, accumulation fp32, master weights fp32 (Adam).
 *
 * Layout: activations channels-last, [z][y][x][c] bf16, x extent 128 (one row
 * of x is one 128-row MMA tile).  Weights [tap][c_out][c_in] bf16, tap =
 * (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1).
 *
 *   k_conv<CIN, COUT, EPI>  implicit-GEMM convolution with tcgen05.mma
 *       (cta_group::1, kind::f16, M = 128 voxels, N = COUT, K = 16 per MMA):
 *       a tile is CONV_ROWS consecutive output rows of one slice; each input
 *       row the tile needs (rows y0 - 1 .. y0 + CONV_ROWS of slices z - 1 ..
 *       z + 1), at each of the three x shifts, is fetched once by a TMA tensor
 *       load (128 x CIN bf16, zero outside the volume) into a ring of
 *       shared-memory stages and feeds every output row it is a tap of (up to
 *       three), 54 boxes per 4 rows instead of 27 per row; the 27 weight tiles
 *       stay in shared memory (one TMA load per CTA); the tile's CONV_ROWS
 *       accumulators live in TMEM, two tiles' worth, so that the epilogue
 *       reads one tile (tcgen05.ld, four epilogue warps) while the next one's
 *       MMAs run.  Warp roles:
 *       warp 0 TMA producer, warp 1 MMA issuer, warps 2-5 epilogue.  Every
 *       mbarrier wait is bounded (about a second); a timeout sets an error
 *       counter and the CTA finishes without further waits.
 *       Epilogues: bias + ReLU to bf16 (hidden layers), residual output in
 *       fp32 (last layer), gradient masked by the layer input's ReLU (input
 *       gradients: the same convolution on dY with the taps mirrored and
 *       c_in / c_out exchanged).
 *   k_conv_wgrad<CIN, COUT>  weight gradients dW[tap][co][ci] = sum_v
 *       X[v + tap][ci] dY[v][co] with tcgen05.mma as well: D[(tap, ci), co] =
 *       A x B^T with A = the shifted inputs (rows (tap, ci), K = voxels) and
 *       B = dY (rows co, K = voxels), both K-major from channel-major copies
 *       (k_wg_shift holds one copy per x shift, so that every TMA box starts
 *       on an aligned x); per 32-voxel chunk the 27 taps' boxes and dY's box
 *       fill a stage, 128 / CIN taps make one M = 128 tile, and the 7 (or 4)
 *       tiles accumulate in TMEM over the CTA's chunks; the epilogue adds the
 *       CTA's partial sums to dW with fp32 atomics.  A row of ones in the
 *       last tile's spare rows gives the bias gradient sum_v dY[v][co].
 *   k_adam, k_publish      Adam on the fp32 master weights, then the bf16
 *       copies in both tap orders.
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cstring>
#include <vector>
#include "pct_device.cuh"
#include "pct_cnn.h" /* include/ */

namespace {

constexpr int CNN_W = 128; /* x extent = MMA M */
constexpr int CNN_LAYERS = 8;
constexpr int CNN_TAPS = 27;
constexpr int CONV_THREADS = 192; /* warp 0 producer, warp 1 MMA, warps 2-5 epilogue */
constexpr int CONV_STAGES = 6;
constexpr int CONV_ROWS = 4;   /* output rows (of 128 voxels) per tile */
constexpr int CONV_ACC = 32;   /* TMEM columns per output row's accumulator (>= COUT) */
constexpr int CONV_TMEM = 2 * CONV_ROWS * CONV_ACC; /* two tiles' accumulators: 256 columns */
enum { EPI_RELU = 0, EPI_OUT = 1, EPI_DGRAD = 2 };

/* (c_in, c_out) of each layer as stored (padded) and as defined */
constexpr int LCIN[CNN_LAYERS] = {16, 32, 32, 32, 32, 32, 32, 32};
constexpr int LCOUT[CNN_LAYERS] = {32, 32, 32, 32, 32, 32, 32, 16};
constexpr int RCIN[CNN_LAYERS] = {2, 32, 32, 32, 32, 32, 32, 32};
constexpr int RCOUT[CNN_LAYERS] = {32, 32, 32, 32, 32, 32, 32, 1};

/* ---- PTX wrappers: mbarrier, TMA, tcgen05 --------------------------------- */
__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(saddr(b)), "r"(parity)
                 : "memory");
    return ok != 0;
}
/* waits for the phase of the given parity; false after about 2^31 SM clocks */
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
    const long long t0 = clock64();
    for (unsigned i = 0;; ++i) {
        if (mbar_try(b, parity)) return true;
        if ((i & 15u) == 15u && clock64() - t0 > (1ll << 31)) return false;
    }
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(saddr(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(saddr(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(saddr(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(saddr(bar))
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
/* whole warp */
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
/* D(tmem) (+)= A(smem) x B(smem)^T: bf16 inputs, fp32 accumulator */
__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
/* arrives once on `bar` when every MMA this thread issued before has completed */
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}
/* 32 TMEM lanes x 16 columns (thread t of the warp: lane base + t) */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

/* Shared-memory matrix descriptor of a K-major tile whose rows are `row_bytes`
 * (32 or 64) long, written by TMA with the matching swizzle (32B or 64B):
 * start address, stride between 8-row groups (8 rows), fixed field 0b001 at
 * bit 46, swizzle mode (6 = 32B, 4 = 64B). */
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, int row_bytes) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16; /* leading offset: unused for swizzled K-major */
    d |= (uint64_t)(((8u * (uint32_t)row_bytes) >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)(row_bytes == 64 ? 4 : 6) << 61;
    return d;
}
/* Instruction descriptor, kind::f16: fp32 D, bf16 A and B, both K-major, M = 128. */
__host__ __device__ constexpr uint32_t umma_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ float bf(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }
__device__ __forceinline__ uint16_t tobf(float f) {
    __nv_bfloat16 b = __float2bfloat16_rn(f);
    return *reinterpret_cast<uint16_t*>(&b);
}

struct ConvArgs {
    int depth, height;       /* z and y extents (x = CNN_W) */
    const float* bias;       /* COUT (padded) fp32, or null */
    uint16_t* out_bf;        /* EPI_RELU / EPI_DGRAD: [v][COUT] bf16 */
    float* out_f;            /* EPI_OUT: [v] fp32 */
    const float* x0;         /* EPI_OUT: residual input [v] */
    const uint16_t* mask;    /* EPI_DGRAD: [v][COUT] bf16 layer input (ReLU mask: > 0) */
    unsigned long long* err; /* timeout counter */
};

template <int CIN, int COUT>
struct ConvSmem {
    static constexpr int ROW = CIN * 2;         /* bytes per A / B row */
    static constexpr int A_BYTES = CNN_W * ROW; /* one stage */
    static constexpr int B_TAP = COUT * ROW;    /* one tap's weights */
    static constexpr int B_BYTES = CNN_TAPS * B_TAP;
    static constexpr int OFF_A = ((B_BYTES + 1023) / 1024) * 1024;
    /* 8 KB after the stages: the MMA's operand reads end well inside the allocation */
    static constexpr int OFF_BAR = OFF_A + CONV_STAGES * A_BYTES + 8192;
    static constexpr int NBAR = 2 * CONV_STAGES + 5; /* full, empty, weights, tmem full x2, tmem empty x2 */
    static constexpr int TOTAL = OFF_BAR + NBAR * 8 + 16 + 1024; /* + TMEM address slot + alignment slack */
};

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(CONV_THREADS, 1) k_conv(const __grid_constant__ CUtensorMap in_map,
                                                          const __grid_constant__ CUtensorMap w_map, ConvArgs p) {
    using L = ConvSmem<CIN, COUT>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t* sB = smem;
    uint8_t* sA = smem + L::OFF_A;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);
    uint64_t* empty = full + CONV_STAGES;
    uint64_t* wbar = empty + CONV_STAGES;
    uint64_t* tfull = wbar + 1;  /* [2]: accumulator buffer b complete */
    uint64_t* tempty = tfull + 2; /* [2]: accumulator buffer b read by the epilogue */
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tempty + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    /* a tile: CONV_ROWS consecutive output rows y0 .. of one slice z */
    const int row_groups = (p.height + CONV_ROWS - 1) / CONV_ROWS;
    const int ntiles = p.depth * row_groups;
    if (threadIdx.x == 0) {
        for (int s = 0; s < CONV_STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(wbar, 1);
        for (int b = 0; b < 2; ++b) {
            mbar_init(tfull + b, 1);
            mbar_init(tempty + b, 4);
        }
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(tslot, CONV_TMEM);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;
    if (warp == 0) {
        if (lane == 0) { /* TMA producer: per tile the input rows y0 - 1 .. y0 + CONV_ROWS of slices
                          * z - 1 .. z + 1, each at the three x shifts, one box each */
            mbar_expect_tx(wbar, (uint32_t)L::B_BYTES);
            tma_load_3d(sB, &w_map, 0, 0, 0, wbar);
            uint32_t it = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int z = t / row_groups, y0 = (t - z * row_groups) * CONV_ROWS;
                for (int dz = -1; dz <= 1 && ok; ++dz)
                    for (int yy = y0 - 1; yy <= y0 + CONV_ROWS && ok; ++yy)
                        for (int dx = -1; dx <= 1; ++dx, ++it) {
                            const int s = (int)(it % CONV_STAGES);
                            const uint32_t round = it / CONV_STAGES;
                            if (round > 0 && !mbar_wait(empty + s, (round - 1) & 1u)) {
                                ok = false;
                                break;
                            }
                            mbar_expect_tx(full + s, (uint32_t)L::A_BYTES);
                            tma_load_4d(sA + s * L::A_BYTES, &in_map, 0, dx, yy, z + dz, full + s);
                        }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) { /* MMA issuer: each box feeds the output rows it is a tap of (up to three) */
            constexpr uint32_t idesc = umma_idesc(COUT);
            /* descriptors of the first stage and the first tap; the others differ only in the
             * start address field (address / 16, all offsets multiples of 16 below 256 KB) */
            const uint64_t da0 = umma_desc(saddr(sA), L::ROW), db0 = umma_desc(saddr(sB), L::ROW);
            ok = mbar_wait(wbar, 0);
            uint32_t it = 0, tile = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++tile) {
                const uint32_t buf = tile & 1u, use = tile >> 1;
                if (use > 0 && !mbar_wait(tempty + buf, (use - 1) & 1u)) { /* the epilogue has read buffer buf */
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t acc0 = tmem + buf * (CONV_ROWS * CONV_ACC);
                const int z = t / row_groups, y0 = (t - z * row_groups) * CONV_ROWS;
                (void)z;
                for (int dz = -1; dz <= 1 && ok; ++dz)
                    for (int yy = y0 - 1; yy <= y0 + CONV_ROWS && ok; ++yy)
                        for (int dx = -1; dx <= 1; ++dx, ++it) {
                            const int s = (int)(it % CONV_STAGES);
                            if (!mbar_wait(full + s, (it / CONV_STAGES) & 1u)) {
                                ok = false;
                                break;
                            }
                            tc_fence_after();
                            const uint64_t da = da0 + (uint64_t)((uint32_t)(s * L::A_BYTES) >> 4);
#pragma unroll
                            for (int j = 0; j < CONV_ROWS; ++j) {
                                const int dy = yy - (y0 + j);
                                if (dy < -1 || dy > 1) continue;
                                const int tap = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
                                const uint64_t db = db0 + (uint64_t)((uint32_t)(tap * L::B_TAP) >> 4);
                                /* the first contribution to row j: dz = dy = dx = -1 */
                                const bool first = dz == -1 && dy == -1 && dx == -1;
#pragma unroll
                                for (int kk = 0; kk < CIN / 16; ++kk) /* K step: 32 bytes = 2 address units */
                                    umma_bf16(acc0 + (uint32_t)(j * CONV_ACC), da + (uint64_t)(2 * kk),
                                              db + (uint64_t)(2 * kk), idesc, (first && kk == 0) ? 0u : 1u);
                            }
                            umma_commit(empty + s); /* the stage is free once these MMAs have read it */
                        }
                if (!ok) break;
                umma_commit(tfull + buf);
            }
        }
    } else { /* epilogue: warps 2-5, TMEM lanes 32 * (warp % 4) .. + 31 */
        const int q = warp & 3;
        const int x = q * 32 + lane; /* the tile's row = voxel x */
        uint32_t tile = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++tile) {
            const uint32_t buf = tile & 1u, use = tile >> 1;
            if (!mbar_wait(tfull + buf, use & 1u)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const int z = t / row_groups, y0 = (t - z * row_groups) * CONV_ROWS;
            for (int j = 0; j < CONV_ROWS; ++j) {
                uint32_t r[32];
                const uint32_t col = buf * (CONV_ROWS * CONV_ACC) + (uint32_t)(j * CONV_ACC);
                tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + col, r);
                if (COUT > 16) tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + col + 16, r + 16);
                tmem_wait_ld();
                const int y = y0 + j;
                if (y >= p.height) continue;
                const size_t v = ((size_t)z * p.height + y) * CNN_W + x;
                if (EPI == EPI_OUT) {
                    p.out_f[v] = p.x0[v] + (__uint_as_float(r[0]) + p.bias[0]);
                } else {
                    uint32_t packed[COUT / 2];
                    if (EPI == EPI_RELU) {
#pragma unroll
                        for (int c = 0; c < COUT; c += 2) {
                            const float a = fmaxf(__uint_as_float(r[c]) + p.bias[c], 0.0f);
                            const float b = fmaxf(__uint_as_float(r[c + 1]) + p.bias[c + 1], 0.0f);
                            packed[c / 2] = (uint32_t)tobf(a) | ((uint32_t)tobf(b) << 16);
                        }
                    } else { /* EPI_DGRAD */
                        const uint4* mrow = reinterpret_cast<const uint4*>(p.mask + v * COUT);
#pragma unroll
                        for (int c8 = 0; c8 < COUT / 8; ++c8) {
                            const uint4 m = mrow[c8];
                            const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
#pragma unroll
                            for (int h = 0; h < 4; ++h) {
                                const int c = c8 * 8 + h * 2;
                                const float a = bf((uint16_t)(mw[h] & 0xffffu)) > 0.0f ? __uint_as_float(r[c]) : 0.0f;
                                const float b = bf((uint16_t)(mw[h] >> 16)) > 0.0f ? __uint_as_float(r[c + 1]) : 0.0f;
                                packed[c / 2] = (uint32_t)tobf(a) | ((uint32_t)tobf(b) << 16);
                            }
                        }
                    }
                    uint4* orow = reinterpret_cast<uint4*>(p.out_bf + v * COUT);
#pragma unroll
                    for (int c8 = 0; c8 < COUT / 8; ++c8)
                        orow[c8] = make_uint4(packed[c8 * 4], packed[c8 * 4 + 1], packed[c8 * 4 + 2], packed[c8 * 4 + 3]);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty + buf);
        }
    }
    if (!ok && lane == 0) atomicAdd(p.err, 1ull);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, CONV_TMEM);
    }
}

/* ---- CUDA-core kernels ---------------------------------------------------- */

/* the network input: [v][16] bf16 = (x0, hull, 0, ...) */
__global__ void k_cnn_pack_input(int64_t nv, const float* __restrict__ x0, const uint8_t* __restrict__ hull,
                                 uint16_t* __restrict__ in) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    uint4* o = reinterpret_cast<uint4*>(in + v * 16);
    o[0] = make_uint4((uint32_t)tobf(x0[v]) | ((uint32_t)tobf(hull[v] ? 1.0f : 0.0f) << 16), 0u, 0u, 0u);
    o[1] = make_uint4(0u, 0u, 0u, 0u);
}

/* loss = sum (out - target)^2 / nv (binary64 sum); dY8[v][0] = 2 (out - target) / nv */
__global__ void k_cnn_loss(int64_t nv, const float* __restrict__ out, const float* __restrict__ target,
                           uint16_t* __restrict__ dy, double* __restrict__ loss) {
    __shared__ double red[8];
    double s = 0.0;
    const float inv = 1.0f / (float)nv;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
        const float d = out[v] - target[v];
        s += (double)d * (double)d;
        if (dy) {
            uint4* o = reinterpret_cast<uint4*>(dy + v * 16);
            o[0] = make_uint4((uint32_t)tobf(2.0f * d * inv), 0u, 0u, 0u);
            o[1] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        atomicAdd(loss, t / (double)nv);
    }
}

/* Channel-major copies of a layer input for the weight gradients:
 * xs[d][c][v] = X[v with x shifted by d - 1][c] (0 outside the volume), d = 0, 1, 2;
 * v = (z * height + y) * 128 + x. */
template <int C>
__global__ void k_wg_shift(int64_t nv, const uint16_t* __restrict__ x, uint16_t* __restrict__ xs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int xx = (int)(i & (CNN_W - 1));
    const int64_t row = i - xx;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int src = xx + d - 1;
        uint32_t w[C / 2];
        if (src >= 0 && src < CNN_W) {
            const uint4* p = reinterpret_cast<const uint4*>(x + (row + src) * C);
#pragma unroll
            for (int k = 0; k < C / 8; ++k) {
                const uint4 u = p[k];
                w[4 * k] = u.x;
                w[4 * k + 1] = u.y;
                w[4 * k + 2] = u.z;
                w[4 * k + 3] = u.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < C / 2; ++k) w[k] = 0u;
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
            xs[((int64_t)d * C + c) * nv + i] = (uint16_t)((c & 1) ? (w[c / 2] >> 16) : (w[c / 2] & 0xffffu));
    }
}

/* dt[c][v] = dY[v][c] */
template <int C>
__global__ void k_wg_dyt(int64_t nv, const uint16_t* __restrict__ dy, uint16_t* __restrict__ dt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const uint4* p = reinterpret_cast<const uint4*>(dy + i * C);
#pragma unroll
    for (int k = 0; k < C / 8; ++k) {
        const uint4 u = p[k];
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            dt[(int64_t)(8 * k + 2 * h) * nv + i] = (uint16_t)(w[h] & 0xffffu);
            dt[(int64_t)(8 * k + 2 * h + 1) * nv + i] = (uint16_t)(w[h] >> 16);
        }
    }
}

constexpr int WG_STAGES = 3;
constexpr int WG_CHUNK = 32; /* voxels of one x row per chunk: K of the stage (64-byte rows) */

template <int CIN, int COUT>
struct WgSmem {
    static constexpr int TPT = 128 / CIN;                      /* taps per M = 128 tile */
    static constexpr int MT = (CNN_TAPS + TPT - 1) / TPT;      /* tiles: 7 (CIN 32) or 4 (CIN 16) */
    static constexpr int A_BOX = CIN * WG_CHUNK * 2;           /* one tap: CIN rows of 64 bytes */
    static constexpr int A_TILE = 128 * WG_CHUNK * 2;          /* 8 KB */
    static constexpr int A_BYTES = MT * A_TILE;                /* the last tile's missing taps: zeros */
    static constexpr int B_BYTES = COUT * WG_CHUNK * 2;
    static constexpr int STAGE = A_BYTES + ((B_BYTES + 1023) / 1024) * 1024;
    static constexpr int OFF_BAR = WG_STAGES * STAGE + 8192;
    static constexpr int NBAR = 2 * WG_STAGES + 1; /* full, empty, tmem full */
    static constexpr int TOTAL = OFF_BAR + NBAR * 8 + 16 + 1024;
    static constexpr int NCOL = MT * COUT;
    static constexpr uint32_t TCOLS = NCOL <= 32 ? 32u : NCOL <= 64 ? 64u : NCOL <= 128 ? 128u : 256u;
};

struct WgArgs {
    int height, chunks, per; /* 4 chunks per x row; this CTA: chunks [blockIdx.x * per, + per) */
    float* dw;               /* [tap][COUT][CIN] fp32, accumulated */
    float* db;               /* [COUT] fp32, accumulated: the bias gradient */
    unsigned long long* err;
};

template <int CIN, int COUT>
__global__ void __launch_bounds__(CONV_THREADS, 1) k_conv_wgrad(const __grid_constant__ CUtensorMap xs_map,
                                                               const __grid_constant__ CUtensorMap dt_map, WgArgs p) {
    using L = WgSmem<CIN, COUT>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);
    uint64_t* empty = full + WG_STAGES;
    uint64_t* tfull = empty + WG_STAGES;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tfull + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c0 = blockIdx.x * p.per;
    const int c1 = c0 + p.per < p.chunks ? c0 + p.per : p.chunks;
    /* the missing taps of the last tile read zeros, except the first row of the first
     * missing tap, which reads ones: its D row is sum_v dY[v][co], the bias gradient
     * (a row of equal values is the same under the 64-byte swizzle) */
    constexpr int PAD = L::A_BYTES - CNN_TAPS * L::A_BOX;
    constexpr uint32_t ONES = 0x3F803F80u; /* two bf16 1.0 */
    for (int st = 0; st < WG_STAGES; ++st)
        for (int k = threadIdx.x; k < PAD / 16; k += CONV_THREADS)
            reinterpret_cast<uint4*>(smem + st * L::STAGE + CNN_TAPS * L::A_BOX)[k] =
                k < 4 ? make_uint4(ONES, ONES, ONES, ONES) : make_uint4(0u, 0u, 0u, 0u);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (threadIdx.x == 0) {
        for (int st = 0; st < WG_STAGES; ++st) {
            mbar_init(full + st, 1);
            mbar_init(empty + st, 1);
        }
        mbar_init(tfull, 1);
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(tslot, L::TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = c1 > c0;
    if (warp == 0) {
        if (lane == 0 && ok) { /* TMA producer */
            uint32_t it = 0;
            for (int c = c0; c < c1; ++c, ++it) {
                const int st = (int)(it % WG_STAGES);
                const uint32_t round = it / WG_STAGES;
                if (round > 0 && !mbar_wait(empty + st, (round - 1) & 1u)) {
                    ok = false;
                    break;
                }
                uint8_t* sa = smem + st * L::STAGE;
                uint8_t* sb = sa + L::A_BYTES;
                const int row = c >> 2, x0 = (c & 3) * WG_CHUNK;
                const int z = row / p.height, y = row - z * p.height;
                mbar_expect_tx(full + st, (uint32_t)(CNN_TAPS * L::A_BOX + L::B_BYTES));
                for (int tap = 0; tap < CNN_TAPS; ++tap) {
                    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
                    tma_load_4d(sa + tap * L::A_BOX, &xs_map, x0, y + dy, z + dz, (dx + 1) * CIN, full + st);
                }
                tma_load_4d(sb, &dt_map, x0, y, z, 0, full + st);
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && ok) { /* MMA issuer */
            constexpr uint32_t idesc = umma_idesc(COUT);
            uint32_t it = 0;
            for (int c = c0; c < c1; ++c, ++it) {
                const int st = (int)(it % WG_STAGES);
                if (!mbar_wait(full + st, (it / WG_STAGES) & 1u)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = saddr(smem + st * L::STAGE), b0 = a0 + L::A_BYTES;
#pragma unroll
                for (int m = 0; m < L::MT; ++m)
#pragma unroll
                    for (int kk = 0; kk < WG_CHUNK / 16; ++kk)
                        umma_bf16(tmem + (uint32_t)(m * COUT), umma_desc(a0 + m * L::A_TILE + kk * 32, 64),
                                  umma_desc(b0 + kk * 32, 64), idesc, (it > 0 || kk > 0) ? 1u : 0u);
                umma_commit(empty + st); /* the stage is free once these MMAs have read it */
            }
            if (ok) umma_commit(tfull);
        }
    } else if (ok) { /* epilogue: warps 2-5, TMEM lanes 32 * (warp % 4) .. + 31 */
        const int q = warp & 3;
        const int r = q * 32 + lane; /* D row: (tap within the tile, c_in) */
        const int tl = r / CIN, ci = r - tl * CIN;
        if (!mbar_wait(tfull, 0)) {
            ok = false;
        } else {
            tc_fence_after();
#pragma unroll 1
            for (int m = 0; m < L::MT; ++m) {
                uint32_t v[32];
                tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(m * COUT), v);
                if (COUT > 16) tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(m * COUT) + 16, v + 16);
                tmem_wait_ld();
                const int tap = m * L::TPT + tl;
                if (tap < CNN_TAPS) {
#pragma unroll
                    for (int co = 0; co < COUT; ++co)
                        atomicAdd(p.dw + ((size_t)tap * COUT + co) * CIN + ci, __uint_as_float(v[co]));
                } else if (tap == CNN_TAPS && ci == 0) { /* the row of ones: the bias gradient */
#pragma unroll
                    for (int co = 0; co < COUT; ++co) atomicAdd(p.db + co, __uint_as_float(v[co]));
                }
            }
            tc_fence_before();
        }
    }
    if (!ok && c1 > c0 && lane == 0 && warp < 6) atomicAdd(p.err, 1ull);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, L::TCOLS);
    }
}

/* Adam (Kingma & Ba 2015) on the fp32 master parameters */
__global__ void k_adam(int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

/* bf16 weights of one layer in both orders from the fp32 master (padded shapes):
 * wf[tap][co][ci] (forward) and wt[26 - tap][ci][co] (input gradients) */
__global__ void k_publish(int cin_r, int cout_r, int cin_p, int cout_p, const float* __restrict__ w,
                          const float* __restrict__ b, uint16_t* __restrict__ wf, uint16_t* __restrict__ wt,
                          float* __restrict__ bias_p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = CNN_TAPS * cin_p * cout_p;
    if (i < cout_p) bias_p[i] = i < cout_r ? b[i] : 0.0f;
    if (i >= n) return;
    const int tap = i / (cin_p * cout_p), rem = i - tap * cin_p * cout_p, co = rem / cin_p, ci = rem - co * cin_p;
    const float val = (co < cout_r && ci < cin_r) ? w[((size_t)tap * cout_r + co) * cin_r + ci] : 0.0f;
    const uint16_t h = tobf(val);
    wf[i] = h;
    if (wt) wt[((size_t)(CNN_TAPS - 1 - tap) * cin_p + ci) * cout_p + co] = h;
}

/* the padded-layout weight gradient of one layer back to the fp32 parameter
 * layout [tap][co][ci] (real sizes) */
__global__ void k_unpad_grad(int cin_r, int cout_r, int cin_p, int cout_p, const float* __restrict__ gp,
                             float* __restrict__ g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= CNN_TAPS * cout_r * cin_r) return;
    const int tap = i / (cout_r * cin_r), rem = i - tap * cout_r * cin_r, co = rem / cin_r, ci = rem - co * cin_r;
    g[i] = gp[((size_t)tap * cout_p + co) * cin_p + ci];
}

/* bf16 [v][C] -> fp32 [v][C] (inspection of activations and gradients) */
__global__ void k_bf_to_f(int64_t n, const uint16_t* __restrict__ a, float* __restrict__ b) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = bf(a[i]);
}

}  // namespace

/* ---- host side ------------------------------------------------------------ */

struct pct_cnn {
    int depth = 0, height = 0, device = 0;
    int64_t nv = 0;
    cudaStream_t stream = nullptr;
    DevBuf in0, act[CNN_LAYERS - 1], out, dy8, dyl[CNN_LAYERS - 1], x0, hull, target;
    DevBuf params, grads, adam_m, adam_v, gpad, bgrad, loss, err, scratch;
    DevBuf wg_x, wg_dy; /* channel-major copies for the weight gradients */
    DevBuf wf[CNN_LAYERS], wt[CNN_LAYERS], bias[CNN_LAYERS];
    CUtensorMap map_in0, map_act[CNN_LAYERS - 1], map_dy8, map_dyl[CNN_LAYERS - 1], map_wf[CNN_LAYERS], map_wt[CNN_LAYERS];
    CUtensorMap map_xs16, map_xs32, map_dt16, map_dt32; /* over wg_x / wg_dy */
    int64_t woff[CNN_LAYERS], boff[CNN_LAYERS], nparams = 0;
    int adam_t = 0;
    int sms = 1;
    int64_t launches = 0;
};

namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

pct_status get_encoder() {
    if (g_encode) return PCT_OK;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
        return pct_fail(PCT_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return PCT_OK;
}

/* [z][y][x][c] bf16 activations: box = one row of x (128 voxels x C channels) */
pct_status make_act_map(CUtensorMap* m, void* ptr, int C, int height, int depth) {
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)CNN_W, (cuuint64_t)height, (cuuint64_t)depth};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)C * 2 * CNN_W, (cuuint64_t)C * 2 * CNN_W * height};
    const cuuint32_t box[4] = {(cuuint32_t)C, (cuuint32_t)CNN_W, 1, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, ptr, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, C == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return pct_fail(PCT_ERR_CUDA, "cuTensorMapEncodeTiled (activations, C=%d): %d", C, (int)r);
    return PCT_OK;
}

/* Channel-major [c][z][y][x] bf16 with `C` channel rows: box = 32 voxels of one x row x `box_c` channels */
pct_status make_cm_map(CUtensorMap* m, void* ptr, int C, int box_c, int height, int depth) {
    const cuuint64_t dims[4] = {(cuuint64_t)CNN_W, (cuuint64_t)height, (cuuint64_t)depth, (cuuint64_t)C};
    const cuuint64_t strides[3] = {(cuuint64_t)CNN_W * 2, (cuuint64_t)CNN_W * 2 * height,
                                   (cuuint64_t)CNN_W * 2 * height * depth};
    const cuuint32_t box[4] = {(cuuint32_t)WG_CHUNK, 1, 1, (cuuint32_t)box_c};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, ptr, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return pct_fail(PCT_ERR_CUDA, "cuTensorMapEncodeTiled (channel-major, C=%d): %d", C, (int)r);
    return PCT_OK;
}

template <int CIN, int COUT>
pct_status launch_wgrad(pct_cnn* n, const uint16_t* x, const uint16_t* dy, const CUtensorMap& xs_map,
                        const CUtensorMap& dt_map) {
    constexpr int smem = WgSmem<CIN, COUT>::TOTAL;
    static bool attr = false;
    if (!attr) {
        PCT_CUDA(cudaFuncSetAttribute(k_conv_wgrad<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    n->launches += 3;
    k_wg_shift<CIN><<<pct_grid_for(n->nv, 256), 256, 0, n->stream>>>(n->nv, x, n->wg_x.as<uint16_t>());
    k_wg_dyt<COUT><<<pct_grid_for(n->nv, 256), 256, 0, n->stream>>>(n->nv, dy, n->wg_dy.as<uint16_t>());
    WgArgs a;
    a.height = n->height;
    a.chunks = n->depth * n->height * (CNN_W / WG_CHUNK);
    const int want = a.chunks < n->sms ? a.chunks : n->sms;
    a.per = (a.chunks + want - 1) / want;
    const int grid = (a.chunks + a.per - 1) / a.per;
    a.dw = n->gpad.as<float>();
    a.db = n->bgrad.as<float>();
    a.err = n->err.as<unsigned long long>();
    k_conv_wgrad<CIN, COUT><<<grid, CONV_THREADS, smem, n->stream>>>(xs_map, dt_map, a);
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

/* [27][N][K] bf16 weights: the whole tensor in one box */
pct_status make_w_map(CUtensorMap* m, void* ptr, int K, int N) {
    const cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)N, (cuuint64_t)CNN_TAPS};
    const cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)K * 2 * N};
    const cuuint32_t box[3] = {(cuuint32_t)K, (cuuint32_t)N, (cuuint32_t)CNN_TAPS};
    const cuuint32_t es[3] = {1, 1, 1};
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, ptr, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, K == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return pct_fail(PCT_ERR_CUDA, "cuTensorMapEncodeTiled (weights %dx%d): %d", N, K, (int)r);
    return PCT_OK;
}

template <int CIN, int COUT, int EPI>
pct_status launch_conv(pct_cnn* n, const CUtensorMap& in, const CUtensorMap& w, const ConvArgs& a) {
    constexpr int smem = ConvSmem<CIN, COUT>::TOTAL;
    static bool attr = false;
    if (!attr) {
        PCT_CUDA(cudaFuncSetAttribute(k_conv<CIN, COUT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr = true;
    }
    const int tiles = n->depth * ((n->height + CONV_ROWS - 1) / CONV_ROWS);
    const int grid = tiles < 2 * n->sms ? tiles : 2 * n->sms;
    ++n->launches;
    k_conv<CIN, COUT, EPI><<<grid, CONV_THREADS, smem, n->stream>>>(in, w, a);
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

ConvArgs conv_args(pct_cnn* n) {
    ConvArgs a;
    memset(&a, 0, sizeof(a));
    a.depth = n->depth;
    a.height = n->height;
    a.err = n->err.as<unsigned long long>();
    return a;
}

const uint16_t* layer_input(pct_cnn* n, int l) { return l == 0 ? n->in0.as<uint16_t>() : n->act[l - 1].as<uint16_t>(); }

pct_status forward(pct_cnn* n) {
    ++n->launches;
    k_cnn_pack_input<<<pct_grid_for(n->nv, 256), 256, 0, n->stream>>>(n->nv, n->x0.as<float>(), n->hull.as<uint8_t>(),
                                                                      n->in0.as<uint16_t>());
    for (int l = 0; l < CNN_LAYERS; ++l) {
        ConvArgs a = conv_args(n);
        a.bias = n->bias[l].as<float>();
        if (l == 0) {
            a.out_bf = n->act[0].as<uint16_t>();
            PCT_TRY((launch_conv<16, 32, EPI_RELU>(n, n->map_in0, n->map_wf[0], a)));
        } else if (l < CNN_LAYERS - 1) {
            a.out_bf = n->act[l].as<uint16_t>();
            PCT_TRY((launch_conv<32, 32, EPI_RELU>(n, n->map_act[l - 1], n->map_wf[l], a)));
        } else {
            a.out_f = n->out.as<float>();
            a.x0 = n->x0.as<float>();
            PCT_TRY((launch_conv<32, 16, EPI_OUT>(n, n->map_act[l - 1], n->map_wf[l], a)));
        }
    }
    return PCT_OK;
}

/* loss and every parameter's gradient (into n->grads) for the current input and
 * target; dY of layer l is the gradient at layer l's output before its ReLU:
 * layer 7 in dy8, layer l < 7 in dyl[l] */
pct_status backward(pct_cnn* n) {
    PCT_CUDA(cudaMemsetAsync(n->loss.p, 0, sizeof(double), n->stream));
    ++n->launches;
    k_cnn_loss<<<2 * n->sms, 256, 0, n->stream>>>(n->nv, n->out.as<float>(), n->target.as<float>(),
                                                  n->dy8.as<uint16_t>(), n->loss.as<double>());
    for (int l = CNN_LAYERS - 1; l >= 0; --l) {
        const uint16_t* dy = l == CNN_LAYERS - 1 ? n->dy8.as<uint16_t>() : n->dyl[l].as<uint16_t>();
        const int cin_p = LCIN[l], cout_p = LCOUT[l];
        PCT_CUDA(cudaMemsetAsync(n->gpad.p, 0, sizeof(float) * CNN_TAPS * cin_p * cout_p, n->stream));
        PCT_CUDA(cudaMemsetAsync(n->bgrad.p, 0, sizeof(float) * 32, n->stream));
        if (l == 0)
            PCT_TRY((launch_wgrad<16, 32>(n, layer_input(n, l), dy, n->map_xs16, n->map_dt32)));
        else if (l == CNN_LAYERS - 1)
            PCT_TRY((launch_wgrad<32, 16>(n, layer_input(n, l), dy, n->map_xs32, n->map_dt16)));
        else
            PCT_TRY((launch_wgrad<32, 32>(n, layer_input(n, l), dy, n->map_xs32, n->map_dt32)));
        ++n->launches;
        const int nw = CNN_TAPS * RCIN[l] * RCOUT[l];
        k_unpad_grad<<<pct_grid_for(nw, 256), 256, 0, n->stream>>>(RCIN[l], RCOUT[l], cin_p, cout_p,
                                                                   n->gpad.as<float>(),
                                                                   n->grads.as<float>() + n->woff[l]);
        PCT_CUDA(cudaMemcpyAsync(n->grads.as<float>() + n->boff[l], n->bgrad.p, sizeof(float) * RCOUT[l],
                                 cudaMemcpyDeviceToDevice, n->stream));
        if (l > 0) { /* dY of layer l - 1 = (W_l^T conv dY_l) masked by layer l's input > 0 */
            ConvArgs a = conv_args(n);
            a.mask = layer_input(n, l);
            a.out_bf = n->dyl[l - 1].as<uint16_t>();
            if (l == CNN_LAYERS - 1)
                PCT_TRY((launch_conv<16, 32, EPI_DGRAD>(n, n->map_dy8, n->map_wt[l], a)));
            else
                PCT_TRY((launch_conv<32, 32, EPI_DGRAD>(n, n->map_dyl[l], n->map_wt[l], a)));
        }
    }
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

pct_status publish(pct_cnn* n) {
    for (int l = 0; l < CNN_LAYERS; ++l) {
        const int cnt = CNN_TAPS * LCIN[l] * LCOUT[l];
        ++n->launches;
        k_publish<<<pct_grid_for(cnt, 256), 256, 0, n->stream>>>(
            RCIN[l], RCOUT[l], LCIN[l], LCOUT[l], n->params.as<float>() + n->woff[l],
            n->params.as<float>() + n->boff[l], n->wf[l].as<uint16_t>(), l > 0 ? n->wt[l].as<uint16_t>() : nullptr,
            n->bias[l].as<float>());
    }
    PCT_CUDA(cudaGetLastError());
    return PCT_OK;
}

pct_status check_err(pct_cnn* n) {
    unsigned long long e = 0;
    PCT_CUDA(cudaMemcpyAsync(&e, n->err.p, sizeof(e), cudaMemcpyDeviceToHost, n->stream));
    PCT_CUDA(cudaStreamSynchronize(n->stream));
    if (e) return pct_fail(PCT_ERR_TIMEOUT, "CNN: %llu tensor-core pipeline waits timed out", e);
    return PCT_OK;
}

/* stages the caller's inputs (host or device) */
pct_status set_inputs(pct_cnn* n, const float* x0, const uint8_t* hull, const float* target, int on_dev) {
    const cudaMemcpyKind k = on_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (x0) PCT_CUDA(cudaMemcpyAsync(n->x0.p, x0, sizeof(float) * n->nv, k, n->stream));
    if (hull) PCT_CUDA(cudaMemcpyAsync(n->hull.p, hull, (size_t)n->nv, k, n->stream));
    if (target) PCT_CUDA(cudaMemcpyAsync(n->target.p, target, sizeof(float) * n->nv, k, n->stream));
    return PCT_OK;
}

uint64_t splitmix(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

}  // namespace

#define CNN_ENTRY(n)                                         \
    if (!(n)) return pct_fail(PCT_ERR_ARGUMENT, "null CNN"); \
    PCT_CUDA(cudaSetDevice((n)->device))

extern "C" size_t pct_cnn_num_params(void) {
    size_t t = 0;
    for (int l = 0; l < CNN_LAYERS; ++l) t += (size_t)CNN_TAPS * RCIN[l] * RCOUT[l] + RCOUT[l];
    return t;
}

extern "C" pct_status pct_cnn_destroy(pct_cnn* n) {
    if (!n) return PCT_OK;
    cudaSetDevice(n->device);
    if (n->stream) cudaStreamSynchronize(n->stream);
    DevBuf* bufs[] = {&n->in0, &n->out, &n->dy8, &n->x0, &n->hull, &n->target, &n->params,
                      &n->grads, &n->adam_m, &n->adam_v, &n->gpad, &n->bgrad, &n->loss, &n->err, &n->scratch,
                      &n->wg_x, &n->wg_dy};
    for (DevBuf* b : bufs) b->release();
    for (int l = 0; l < CNN_LAYERS; ++l) {
        n->wf[l].release();
        n->wt[l].release();
        n->bias[l].release();
        if (l < CNN_LAYERS - 1) {
            n->act[l].release();
            n->dyl[l].release();
        }
    }
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
    return PCT_OK;
}

extern "C" pct_status pct_cnn_create(int device, int depth, int height, int width, pct_cnn** out) {
    if (!out) return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_create: null output");
    *out = nullptr;
    if (width != CNN_W) return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_create: the x extent must be %d, not %d", CNN_W, width);
    if (depth < 1 || height < 1 || (int64_t)depth * height > (1 << 20))
        return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_create: bad volume %d x %d", depth, height);
    PCT_CUDA(cudaSetDevice(device));
    PCT_TRY(get_encoder());
    pct_cnn* n = new pct_cnn();
    n->device = device;
    n->depth = depth;
    n->height = height;
    n->nv = (int64_t)depth * height * CNN_W;
    auto fail = [&](pct_status s) {
        pct_cnn_destroy(n);
        return s;
    };
    if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(pct_fail(PCT_ERR_CUDA, "pct_cnn_create: stream"));
    cudaDeviceGetAttribute(&n->sms, cudaDevAttrMultiProcessorCount, device);
    if (n->sms < 1) n->sms = 1;
    const size_t nv = (size_t)n->nv;
    int64_t off = 0;
    for (int l = 0; l < CNN_LAYERS; ++l) {
        n->woff[l] = off;
        off += (int64_t)CNN_TAPS * RCIN[l] * RCOUT[l];
        n->boff[l] = off;
        off += RCOUT[l];
    }
    n->nparams = off;
    const size_t P = (size_t)off;
    pct_status st = n->in0.alloc(nv * 16 * 2);
    for (int l = 0; l < CNN_LAYERS - 1 && st == PCT_OK; ++l) st = n->act[l].alloc(nv * 32 * 2);
    if (st == PCT_OK) st = n->out.alloc(nv * 4);
    if (st == PCT_OK) st = n->dy8.alloc(nv * 16 * 2);
    for (int l = 0; l < CNN_LAYERS - 1 && st == PCT_OK; ++l) st = n->dyl[l].alloc(nv * 32 * 2);
    if (st == PCT_OK) st = n->x0.alloc(nv * 4);
    if (st == PCT_OK) st = n->hull.alloc(nv);
    if (st == PCT_OK) st = n->target.alloc(nv * 4);
    if (st == PCT_OK) st = n->params.alloc(P * 4);
    if (st == PCT_OK) st = n->grads.alloc(P * 4);
    if (st == PCT_OK) st = n->adam_m.alloc(P * 4);
    if (st == PCT_OK) st = n->adam_v.alloc(P * 4);
    if (st == PCT_OK) st = n->gpad.alloc((size_t)CNN_TAPS * 32 * 32 * 4);
    if (st == PCT_OK) st = n->bgrad.alloc(32 * 4);
    if (st == PCT_OK) st = n->loss.alloc(8);
    if (st == PCT_OK) st = n->err.alloc(8);
    if (st == PCT_OK) st = n->scratch.alloc(nv * 32 * 4);
    if (st == PCT_OK) st = n->wg_x.alloc(nv * 3 * 32 * 2);
    if (st == PCT_OK) st = n->wg_dy.alloc(nv * 32 * 2);
    for (int l = 0; l < CNN_LAYERS && st == PCT_OK; ++l) {
        st = n->wf[l].alloc((size_t)CNN_TAPS * LCIN[l] * LCOUT[l] * 2);
        if (st == PCT_OK && l > 0) st = n->wt[l].alloc((size_t)CNN_TAPS * LCIN[l] * LCOUT[l] * 2);
        if (st == PCT_OK) st = n->bias[l].alloc(32 * 4);
    }
    if (st != PCT_OK) return fail(st);
    if (cudaMemsetAsync(n->params.p, 0, P * 4, n->stream) != cudaSuccess ||
        cudaMemsetAsync(n->adam_m.p, 0, P * 4, n->stream) != cudaSuccess ||
        cudaMemsetAsync(n->adam_v.p, 0, P * 4, n->stream) != cudaSuccess ||
        cudaMemsetAsync(n->err.p, 0, 8, n->stream) != cudaSuccess)
        return fail(pct_fail(PCT_ERR_CUDA, "pct_cnn_create: memset"));
    st = make_act_map(&n->map_in0, n->in0.p, 16, height, depth);
    for (int l = 0; l < CNN_LAYERS - 1 && st == PCT_OK; ++l)
        st = make_act_map(&n->map_act[l], n->act[l].p, 32, height, depth);
    if (st == PCT_OK) st = make_act_map(&n->map_dy8, n->dy8.p, 16, height, depth);
    for (int l = 0; l < CNN_LAYERS - 1 && st == PCT_OK; ++l)
        st = make_act_map(&n->map_dyl[l], n->dyl[l].p, 32, height, depth);
    for (int l = 0; l < CNN_LAYERS && st == PCT_OK; ++l) {
        st = make_w_map(&n->map_wf[l], n->wf[l].p, LCIN[l], LCOUT[l]);
        if (st == PCT_OK && l > 0) st = make_w_map(&n->map_wt[l], n->wt[l].p, LCOUT[l], LCIN[l]);
    }
    if (st == PCT_OK) st = make_cm_map(&n->map_xs16, n->wg_x.p, 3 * 16, 16, height, depth);
    if (st == PCT_OK) st = make_cm_map(&n->map_xs32, n->wg_x.p, 3 * 32, 32, height, depth);
    if (st == PCT_OK) st = make_cm_map(&n->map_dt16, n->wg_dy.p, 16, 16, height, depth);
    if (st == PCT_OK) st = make_cm_map(&n->map_dt32, n->wg_dy.p, 32, 32, height, depth);
    if (st == PCT_OK) st = publish(n);
    if (st == PCT_OK && cudaStreamSynchronize(n->stream) != cudaSuccess) st = pct_fail(PCT_ERR_CUDA, "pct_cnn_create");
    if (st != PCT_OK) return fail(st);
    *out = n;
    return PCT_OK;
}

extern "C" pct_status pct_cnn_init(pct_cnn* n, uint64_t seed) {
    CNN_ENTRY(n);
    std::vector<float> w((size_t)n->nparams, 0.0f);
    uint64_t s = seed;
    for (int l = 0; l < CNN_LAYERS; ++l) {
        /* He-uniform for the ReLU layers; the last layer starts at zero (the net starts as x0) */
        const double bound = l < CNN_LAYERS - 1 ? sqrt(6.0 / (CNN_TAPS * RCIN[l])) : 0.0;
        const int64_t cnt = (int64_t)CNN_TAPS * RCIN[l] * RCOUT[l];
        for (int64_t i = 0; i < cnt; ++i) {
            const double u = ((double)(splitmix(&s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            w[(size_t)(n->woff[l] + i)] = (float)((2.0 * u - 1.0) * bound);
        }
    }
    PCT_CUDA(cudaMemcpyAsync(n->params.p, w.data(), w.size() * 4, cudaMemcpyHostToDevice, n->stream));
    PCT_CUDA(cudaMemsetAsync(n->adam_m.p, 0, w.size() * 4, n->stream));
    PCT_CUDA(cudaMemsetAsync(n->adam_v.p, 0, w.size() * 4, n->stream));
    n->adam_t = 0;
    PCT_TRY(publish(n));
    PCT_CUDA(cudaStreamSynchronize(n->stream));
    return PCT_OK;
}

extern "C" pct_status pct_cnn_set_params(pct_cnn* n, const float* host, size_t count) {
    CNN_ENTRY(n);
    if (!host || count != (size_t)n->nparams)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_set_params: need %lld values", (long long)n->nparams);
    PCT_CUDA(cudaMemcpyAsync(n->params.p, host, count * 4, cudaMemcpyHostToDevice, n->stream));
    PCT_TRY(publish(n));
    PCT_CUDA(cudaStreamSynchronize(n->stream));
    return PCT_OK;
}

extern "C" pct_status pct_cnn_get_params(pct_cnn* n, float* host, size_t count) {
    CNN_ENTRY(n);
    if (!host || count != (size_t)n->nparams)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_get_params: need %lld values", (long long)n->nparams);
    PCT_CUDA(cudaMemcpyAsync(host, n->params.p, count * 4, cudaMemcpyDeviceToHost, n->stream));
    PCT_CUDA(cudaStreamSynchronize(n->stream));
    return PCT_OK;
}

extern "C" pct_status pct_cnn_forward(pct_cnn* n, const float* x0, const uint8_t* hull, float* out, int on_dev) {
    CNN_ENTRY(n);
    if (!x0 || !hull || !out) return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_forward: null argument");
    PCT_TRY(set_inputs(n, x0, hull, nullptr, on_dev));
    PCT_TRY(forward(n));
    PCT_CUDA(cudaMemcpyAsync(out, n->out.p, sizeof(float) * n->nv,
                             on_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, n->stream));
    return check_err(n);
}

extern "C" pct_status pct_cnn_gradients(pct_cnn* n, const float* x0, const uint8_t* hull, const float* target,
                                        int on_dev, double* loss, float* grads_host) {
    CNN_ENTRY(n);
    if (!x0 || !hull || !target) return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_gradients: null argument");
    PCT_TRY(set_inputs(n, x0, hull, target, on_dev));
    PCT_TRY(forward(n));
    PCT_TRY(backward(n));
    if (loss) PCT_CUDA(cudaMemcpyAsync(loss, n->loss.p, sizeof(double), cudaMemcpyDeviceToHost, n->stream));
    if (grads_host)
        PCT_CUDA(cudaMemcpyAsync(grads_host, n->grads.p, sizeof(float) * n->nparams, cudaMemcpyDeviceToHost, n->stream));
    return check_err(n);
}

extern "C" pct_status pct_cnn_train_step(pct_cnn* n, const float* x0, const uint8_t* hull, const float* target,
                                         int on_dev, float lr, double* loss) {
    CNN_ENTRY(n);
    if (!x0 || !hull || !target) return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_train_step: null argument");
    PCT_TRY(set_inputs(n, x0, hull, target, on_dev));
    PCT_TRY(forward(n));
    PCT_TRY(backward(n));
    ++n->adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)n->adam_t), c2 = 1.0f - powf(b2, (float)n->adam_t);
    ++n->launches;
    k_adam<<<pct_grid_for(n->nparams, 256), 256, 0, n->stream>>>(n->nparams, n->params.as<float>(), n->grads.as<float>(),
                                                                 n->adam_m.as<float>(), n->adam_v.as<float>(), lr, b1,
                                                                 b2, 1e-8f, c1, c2);
    PCT_CUDA(cudaGetLastError());
    PCT_TRY(publish(n));
    if (loss) PCT_CUDA(cudaMemcpyAsync(loss, n->loss.p, sizeof(double), cudaMemcpyDeviceToHost, n->stream));
    return check_err(n);
}

extern "C" pct_status pct_cnn_inspect(pct_cnn* n, int kind, int layer, float* host, size_t count) {
    CNN_ENTRY(n);
    const uint16_t* src = nullptr;
    int C = 32;
    if (kind == 0 && layer >= 0 && layer < CNN_LAYERS - 1) src = n->act[layer].as<uint16_t>();
    if (kind == 1 && layer == CNN_LAYERS - 1) {
        src = n->dy8.as<uint16_t>();
        C = 16;
    }
    if (kind == 1 && layer >= 0 && layer < CNN_LAYERS - 1) src = n->dyl[layer].as<uint16_t>();
    if (!src || !host || count != (size_t)n->nv * C) return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_inspect: bad request");
    k_bf_to_f<<<pct_grid_for(n->nv * C, 256), 256, 0, n->stream>>>(n->nv * C, src, n->scratch.as<float>());
    PCT_CUDA(cudaGetLastError());
    PCT_CUDA(cudaMemcpyAsync(host, n->scratch.p, count * 4, cudaMemcpyDeviceToHost, n->stream));
    PCT_CUDA(cudaStreamSynchronize(n->stream));
    return PCT_OK;
}

extern "C" pct_status pct_cnn_counts(pct_cnn* n, int64_t* kernel_launches) {
    CNN_ENTRY(n);
    if (kernel_launches) *kernel_launches = n->launches;
    return PCT_OK;
}

extern "C" pct_status pct_cnn_warm_start(pct_ctx* c, pct_cnn* n) {
    if (!c) return pct_fail(PCT_ERR_ARGUMENT, "null context");
    CNN_ENTRY(n);
    if (c->stage < ST_X0) return pct_fail(PCT_ERR_STATE, "pct_cnn_warm_start needs define_initial_iterate");
    if (c->geo.columns != CNN_W || c->geo.rows != n->height || c->geo.slices != n->depth)
        return pct_fail(PCT_ERR_ARGUMENT, "pct_cnn_warm_start: the network is %dx%dx%d, the image %dx%dx%d", CNN_W,
                        n->height, n->depth, c->geo.columns, c->geo.rows, c->geo.slices);
    PCT_CUDA(cudaStreamSynchronize(c->stream));
    PCT_TRY(set_inputs(n, c->x0.as<float>(), c->x_hull_filtered.as<uint8_t>(), nullptr, 1));
    PCT_TRY(forward(n));
    PCT_CUDA(cudaMemcpyAsync(c->x0.p, n->out.p, sizeof(float) * n->nv, cudaMemcpyDeviceToDevice, n->stream));
    PCT_CUDA(cudaMemcpyAsync(c->x.p, n->out.p, sizeof(float) * n->nv, cudaMemcpyDeviceToDevice, n->stream));
    return check_err(n);
}
