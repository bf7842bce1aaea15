/*
 * dct_tc.cu -- dctimestep's product on the 5th-generation tensor cores,
 * BF16x3 split precision with FP32 accumulation.
 *
 * R[m,n,c] = sum_k A[m,k,c] * B[k,n,c] for each colour channel c
 * (util/cmatrix.c:421-474 cm_multiply; the channels do not mix).  Each FP32
 * operand x is split as x = hi + lo + r with hi = bf16(x), lo = bf16(x - hi),
 * |r| <= 2^-18 |x|, and the product is formed as hi*hi + hi*lo + lo*hi: three
 * BF16 tensor-core products accumulating in FP32 in tensor memory (the lo*lo
 * term is below the FP32 rounding of the sum).
 *
 * 1. k_split_a / k_split_b (memory bound) de-interleave the RGB operands
 *    into bf16 hi/lo planes, K contiguous, zero padded to the tile sizes:
 *    As[c][h][Mp][Kp] and Bs[c][h][Np][Kp] (B transposed through shared
 *    memory).
 * 2. k_dct_tc: a persistent kernel, one CTA per SM, 10 warps:
 *      warp 0  TMA producer: 128x64 (A) and 256x64 (B) bf16 boxes with the
 *              128-byte swizzle, hi and lo, into a 2-stage ring (96 KB/stage)
 *      warp 1  allocates 512 TMEM columns (two 128x256 FP32 accumulators)
 *              and one lane issues tcgen05.mma (M=128, N=256, K=16, 12 per
 *              64-wide K block), committing each stage back to the producer
 *              and each finished K chunk (256 of K) to the epilogue
 *      warps 2-9  epilogue: tcgen05.ld of a finished chunk (each warp its
 *              32-lane TMEM sub-partition and one half of the columns) into
 *              FP32 registers, then the interleaved RGB store of the tile.
 *              The FP32 accumulation inside the tensor cores is biased:
 *              its error grows linearly with the number of products in one
 *              accumulator (measured, with all of K in one accumulator:
 *              mean relative error 3.2e-6 at K = 700, 1.2e-5 at K = 2306).
 *              Summing chunks of 48 products in registers with IEEE
 *              rounding bounds that growth.  The two accumulators alternate,
 *              so the epilogue of one chunk overlaps the products of the
 *              next.
 *    Tiles run channel-innermost, so the three channels of one output block
 *    are written at the same time by neighbouring CTAs and merge in L2, and
 *    in groups of 16 row tiles for operand reuse in L2.
 *
 * Every wait on an mbarrier is bounded (two seconds of %globaltimer); on
 * expiry the CTA records an error code, stops issuing work, waits (bounded)
 * for its copies and products in flight and frees its tensor memory, and
 * the host reports GB_ECUDA.
 */
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "dct.h"
#include "../../include/gbrad.h"

namespace {

constexpr int TM = 128, TN = 256, TK = 64;          /* tile; TK bf16 = 128 bytes */
constexpr int STAGES = 2;
constexpr int A_BYTES = TM * TK * 2;                /* 16 KB */
constexpr int B_BYTES = TN * TK * 2;                /* 32 KB */
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr int TMEM_COLS = 512;                      /* 2 accumulators x TN */
constexpr int GROUP_M = 16;                         /* row tiles per raster group */
constexpr int NTHREADS = 320;                       /* producer, MMA, 8 epilogue warps */
constexpr int CHUNK_KB = 4;                         /* K blocks per accumulator chunk (K = 256) */
constexpr int EPI_COLS = TN / 2;                    /* columns per epilogue thread */
constexpr uint64_t WAIT_NS = 2000000000ull;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /* alignment */ + 256 /* barriers */;

/* tcgen05 instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B
 * BF16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit
 * 17, M >> 4 at bit 24 */
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                           ((uint32_t)(TM >> 4) << 24);

enum { ERR_NONE = 0, ERR_FULL = 1, ERR_EMPTY = 2, ERR_TFULL = 3, ERR_TEMPTY = 4, ERR_DRAIN = 5 };

struct Shape {
    int M, K, N;          /* true sizes */
    int Mp, Kp, Np;       /* padded to TM, TK, TN */
    int mt, nt, kb;       /* tile counts, K blocks */
    long long tiles;      /* mt * nt * 3 */
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

/* Wait for the phase of `parity` to complete, at most WAIT_NS.  With
 * `respect_abort`, give up at once when the CTA has aborted. */
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err, int code,
                          bool respect_abort = true)
{
    if (mbar_try(bar, parity))
        return true;
    uint64_t t0 = globaltimer();
    for (;;) {
        if (respect_abort && *abort_flag)
            return false;
        if (mbar_try(bar, parity))
            return true;
        if (globaltimer() - t0 > WAIT_NS) {
            *abort_flag = 1;
            atomicCAS(err, 0, code);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

/* shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
 * 1024 bytes apart (stride byte offset), descriptor version 1 (bit 46) */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t dt, uint64_t a, uint64_t b, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(dt), "l"(a), "l"(b), "r"(IDESC), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = __uint_as_float(r[i]);
}

/* tile t -> (channel, row tile, column tile): channel innermost, then row
 * tiles in groups of GROUP_M sweeping the column tiles */
__device__ __forceinline__ void tile_coords(const Shape &s, long long t, int &c, int &mi, int &ni)
{
    c = (int)(t % 3);
    long long u = t / 3;
    long long per_group = (long long)GROUP_M * s.nt;
    int g = (int)(u / per_group);
    int r = (int)(u % per_group);
    int gm = s.mt - g * GROUP_M;
    if (gm > GROUP_M)
        gm = GROUP_M;
    mi = g * GROUP_M + r % gm;
    ni = r / gm;
}

__global__ void __launch_bounds__(NTHREADS, 1)
k_dct_tc(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, Shape s,
         float *__restrict__ C, int *err)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + STAGES * STAGE_BYTES);
    /* bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], drain */
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES;
    const uint32_t tfull0 = empty0 + 8 * STAGES, tempty0 = tfull0 + 16, drain = tempty0 + 16;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * STAGES + 5);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; i++) {
            mbar_init(full0 + 8 * i, 1);
            mbar_init(empty0 + 8 * i, 1);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(tfull0 + 8 * i, 1);
            mbar_init(tempty0 + 8 * i, 8 * 32);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        /* ---------------- TMA producer */
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapA) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapB) : "memory");
            long long it = 0;
            for (long long t = blockIdx.x; t < s.tiles && !*abort_flag; t += gridDim.x) {
                int c, mi, ni;
                tile_coords(s, t, c, mi, ni);
                const int ya = 2 * c * s.Mp + mi * TM, yb = 2 * c * s.Np + ni * TN;
                for (int kb = 0; kb < s.kb; kb++, it++) {
                    const int st = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                    if (!mbar_wait(empty0 + 8 * st, ph ^ 1, abort_flag, err, ERR_EMPTY))
                        break;
                    const uint32_t base = smem_u32(smem + st * STAGE_BYTES), fb = full0 + 8 * st;
                    mbar_expect_tx(fb, STAGE_BYTES);
                    tma_load_2d(base, &mapA, kb * TK, ya, fb);
                    tma_load_2d(base + A_BYTES, &mapA, kb * TK, ya + s.Mp, fb);
                    tma_load_2d(base + 2 * A_BYTES, &mapB, kb * TK, yb, fb);
                    tma_load_2d(base + 2 * A_BYTES + B_BYTES, &mapB, kb * TK, yb + s.Np, fb);
                }
            }
            /* copies in flight land before the CTA can exit */
            for (long long j = it - STAGES; j < it; j++) {
                if (j < 0)
                    continue;
                mbar_wait(full0 + 8 * (int)(j % STAGES), (uint32_t)((j / STAGES) & 1), abort_flag, err, ERR_FULL,
                          false);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        /* ---------------- MMA issuer */
        if (lane == 0) {
            long long it = 0, cl = 0;
            bool ok = true;
            for (long long t = blockIdx.x; t < s.tiles && ok; t += gridDim.x) {
                for (int k0 = 0; k0 < s.kb && ok; k0 += CHUNK_KB, cl++) {
                    const int buf = (int)(cl & 1);
                    const uint32_t use = (uint32_t)((cl >> 1) & 1);
                    if (!mbar_wait(tempty0 + 8 * buf, use ^ 1, abort_flag, err, ERR_TEMPTY)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dt = tmem + (uint32_t)(buf * TN);
                    const int k1 = k0 + CHUNK_KB < s.kb ? k0 + CHUNK_KB : s.kb;
                    for (int kb = k0; kb < k1; kb++, it++) {
                        const int st = (int)(it % STAGES);
                        const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                        if (!mbar_wait(full0 + 8 * st, ph, abort_flag, err, ERR_FULL)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t base = smem_u32(smem + st * STAGE_BYTES);
#pragma unroll
                        for (int j = 0; j < TK / 16; j++) {
                            const uint64_t ahi = sdesc(base + 32 * j), alo = sdesc(base + A_BYTES + 32 * j);
                            const uint64_t bhi = sdesc(base + 2 * A_BYTES + 32 * j);
                            const uint64_t blo = sdesc(base + 2 * A_BYTES + B_BYTES + 32 * j);
                            mma_bf16(dt, ahi, bhi, (kb != k0) | (j != 0));
                            mma_bf16(dt, ahi, blo, 1);
                            mma_bf16(dt, alo, bhi, 1);
                        }
                        mma_commit(empty0 + 8 * st);      /* stage free once these products finish */
                    }
                    if (ok)
                        mma_commit(tfull0 + 8 * buf);     /* chunk complete */
                }
            }
            /* every product issued has finished before tensor memory is freed */
            mma_commit(drain);
            mbar_wait(drain, 0, abort_flag, err, ERR_DRAIN, false);
        }
        __syncwarp();
    } else {
        /* ---------------- epilogue: warps 2..9; TMEM sub-partition warp % 4,
         * column half (warp - 2) / 4.  Each K chunk's FP32 accumulator is
         * added into registers (IEEE round to nearest), so the tensor cores'
         * accumulation rounding acts on chains of CHUNK_KB * 12 products only */
        const int sub = warp & 3, half = (warp - 2) >> 2;
        long long cl = 0;
        bool ok = true;
        for (long long t = blockIdx.x; t < s.tiles && ok; t += gridDim.x) {
            float acc[EPI_COLS];
#pragma unroll
            for (int i = 0; i < EPI_COLS; i++)
                acc[i] = 0.f;
            for (int k0 = 0; k0 < s.kb; k0 += CHUNK_KB, cl++) {
                const int buf = (int)(cl & 1);
                const uint32_t use = (uint32_t)((cl >> 1) & 1);
                ok = mbar_wait(tfull0 + 8 * buf, use, abort_flag, err, ERR_TFULL);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok)
                    break;
                tc_fence_after();
                const uint32_t tb = tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)(buf * TN + half * EPI_COLS);
#pragma unroll
                for (int cb = 0; cb < EPI_COLS; cb += 16) {
                    float v[16];
                    tmem_ld16(tb + (uint32_t)cb, v);
#pragma unroll
                    for (int i = 0; i < 16; i++)
                        acc[cb + i] += v[i];
                }
                tc_fence_before();
                mbar_arrive(tempty0 + 8 * buf);
            }
            if (!ok)
                break;
            int c, mi, ni;
            tile_coords(s, t, c, mi, ni);
            const int m = mi * TM + sub * 32 + lane;
            if (m < s.M) {
                float *row = C + ((long long)m * s.N) * 3 + c;
                const int n0 = ni * TN + half * EPI_COLS;
#pragma unroll
                for (int i = 0; i < EPI_COLS; i++) {
                    const int n = n0 + i;
                    if (n < s.N)
                        row[3LL * n] = acc[i];
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
}

/* A[m][k][c] (interleaved RGB) -> As[c][h][Mp][Kp] bf16 hi/lo, one thread
 * per element of the padded plane (zeros in the padding) */
__global__ void k_split_a(const float *__restrict__ A, __nv_bfloat16 *__restrict__ As, int M, int K, int Mp,
                          int Kp)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)Mp * Kp)
        return;
    const int m = (int)(i / Kp), k = (int)(i % Kp);
    const bool in = m < M && k < K;
    const size_t plane = (size_t)Mp * Kp;
    const float *a = in ? A + 3 * ((long long)m * K + k) : A;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float x = in ? a[c] : 0.f;
        const __nv_bfloat16 hi = __float2bfloat16_rn(x);
        const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
        As[(2 * c) * plane + i] = hi;
        As[(2 * c + 1) * plane + i] = lo;
    }
}

/* B[k][n][c] -> Bs[c][h][Np][Kp] (transposed, K contiguous) through a 32x32
 * shared tile per channel; the grid covers the padded plane */
__global__ void k_split_b(const float *__restrict__ B, __nv_bfloat16 *__restrict__ Bs, int K, int N, int Np,
                          int Kp)
{
    __shared__ float tile[3][32][33];
    const int k0 = blockIdx.y * 32, n0 = blockIdx.x * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;          /* 32 x 8 */
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r;
        for (int q = tx; q < 96; q += 32) {
            const int n = n0 + q / 3, c = q % 3;
            tile[c][r][q / 3] = (k < K && n < N) ? B[((size_t)k * N + n) * 3 + c] : 0.f;
        }
    }
    __syncthreads();
    const size_t plane = (size_t)Np * Kp;
    for (int r = ty; r < 32; r += 8) {            /* padded plane: zeros beyond K, N */
        const int n = n0 + r, k = k0 + tx;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float x = tile[c][tx][r];
            const __nv_bfloat16 hi = __float2bfloat16_rn(x);
            const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
            Bs[(2 * c) * plane + (size_t)n * Kp + k] = hi;
            Bs[(2 * c + 1) * plane + (size_t)n * Kp + k] = lo;
        }
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

/* rows x Kp bf16 matrix, box TK x box_rows, 128-byte swizzle */
bool make_map(CUtensorMap *m, const void *base, uint64_t rows, uint64_t kp, uint32_t box_rows)
{
    auto fn = encode_fn();
    if (!fn)
        return false;
    cuuint64_t dims[2] = {kp, rows};
    cuuint64_t strides[1] = {kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)TK, box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int gb_dct_bf16x3(const float *A, const float *B, int64_t M, int64_t K, int64_t N, float *C, cudaStream_t st,
                  std::string &err)
{
    auto rnd = [](int64_t x, int64_t q) { return (x + q - 1) / q * q; };
    if (M > (1 << 24) || K > (1 << 20) || N > (1 << 24) || M * K > (1ll << 37) || K * N > (1ll << 37)) {
        err = "matrix too large for the BF16x3 path";
        return GB_EINVAL;
    }
    Shape s;
    s.M = (int)M;
    s.K = (int)K;
    s.N = (int)N;
    s.Mp = (int)rnd(M, TM);
    s.Kp = (int)rnd(K, TK);
    s.Np = (int)rnd(N, TN);
    s.mt = s.Mp / TM;
    s.nt = s.Np / TN;
    s.kb = s.Kp / TK;
    s.tiles = (long long)s.mt * s.nt * 3;
    const size_t a_elems = (size_t)6 * s.Mp * s.Kp, b_elems = (size_t)6 * s.Np * s.Kp;
    /* workspace (error flag, split A, split B), kept per device between
     * calls and grown on demand; calls are serialised on it */
    const size_t a_off = 256, b_off = a_off + ((a_elems * 2 + 255) & ~(size_t)255);
    const size_t total = b_off + b_elems * 2;
    static std::mutex lock;
    static unsigned char *ws_dev[64];
    static size_t ws_size[64];
    std::lock_guard<std::mutex> guard(lock);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        err = "no usable CUDA device";
        return GB_ECUDA;
    }
    if (ws_size[dev] < total) {
        if (ws_dev[dev]) {
            cudaStreamSynchronize(st);
            cudaFree(ws_dev[dev]);
        }
        ws_dev[dev] = nullptr;
        ws_size[dev] = 0;
        if (cudaMalloc(&ws_dev[dev], total) != cudaSuccess) {
            cudaGetLastError();
            ws_dev[dev] = nullptr;
            err = "cannot allocate the BF16x3 operand planes";
            return GB_ENOMEM;
        }
        ws_size[dev] = total;
    }
    unsigned char *ws = ws_dev[dev];
    int *d_err = (int *)ws;
    __nv_bfloat16 *As = (__nv_bfloat16 *)(ws + a_off), *Bs = (__nv_bfloat16 *)(ws + b_off);
    int rc = GB_OK;
    CUtensorMap ma, mb;
    do {
        if (cudaMemsetAsync(d_err, 0, sizeof(int), st) != cudaSuccess) {
            err = "memset failed";
            rc = GB_ECUDA;
            break;
        }
        const long long na = (long long)s.Mp * s.Kp;
        k_split_a<<<(unsigned)((na + 255) / 256), 256, 0, st>>>(A, As, s.M, s.K, s.Mp, s.Kp);
        k_split_b<<<dim3((unsigned)(s.Np / 32), (unsigned)(s.Kp / 32)), dim3(32, 8), 0, st>>>(B, Bs, s.K, s.N,
                                                                                           s.Np, s.Kp);
        if (!make_map(&ma, As, (uint64_t)6 * s.Mp, (uint64_t)s.Kp, TM) ||
            !make_map(&mb, Bs, (uint64_t)6 * s.Np, (uint64_t)s.Kp, TN)) {
            err = "cannot encode the TMA tensor maps";
            rc = GB_ECUDA;
            break;
        }
        static int sms = 0;
        if (!sms) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (cudaFuncSetAttribute(k_dct_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) !=
                cudaSuccess) {
                sms = 0;
                err = "cannot reserve shared memory for the tensor-core kernel";
                rc = GB_ECUDA;
                break;
            }
        }
        const long long grid = s.tiles < sms ? s.tiles : sms;
        k_dct_tc<<<(unsigned)grid, NTHREADS, SMEM_BYTES, st>>>(ma, mb, s, C, d_err);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            err = cudaGetErrorString(e);
            rc = GB_ECUDA;
            break;
        }
        int h_err = 0;
        if (cudaMemcpyAsync(&h_err, d_err, sizeof h_err, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            err = cudaGetErrorString(cudaGetLastError());
            rc = GB_ECUDA;
            break;
        }
        if (h_err) {
            err = "tensor-core pipeline wait expired (code " + std::to_string(h_err) + ")";
            rc = GB_ECUDA;
        }
    } while (0);
    return rc;
}
