/*
 * dct_tc.cu -- dctimestep's product on the 5th-generation tensor cores.
 *
 * R[m,n,c] = sum_k A[m,k,c] * B[k,n,c] for each colour channel c
 * (util/cmatrix.c:421-474 cm_multiply; the channels do not mix), with the
 * reference's skip of all-zero rows of A and all-zero columns of B (a row
 * or column is zero when every byte of its colours is, cmatrix.c:435-450):
 * their outputs are written as zeros and the product runs over the others
 * only.  Three arithmetic forms share one kernel:
 *
 *   BF16X3  x = hi + lo + r, hi = bf16(x), lo = bf16(x - hi), |r| <= 2^-16 |x|;
 *           product hi*hi + hi*lo + lo*hi (three bf16 products).  The
 *           residual of the two-term split bounds the error of one product
 *           at about 2^-15 relative: an output dominated by one product (a
 *           sun patch) can be off by 2e-5.
 *   FP16X3  every row of A and every column of B is first scaled by a power
 *           of two that brings its largest magnitude (per channel) into
 *           [2^14, 2^15), inside the FP16 range; then x = hi + lo + r with
 *           hi = f16(x), lo = f16(x - hi), |r| <= 2^-22 |x| for all but the
 *           smallest elements of a row (below 2^-16 of its maximum, where
 *           lo becomes subnormal), and the product is hi*hi + hi*lo + lo*hi
 *           (three fp16 products, exact in the FP32 accumulator).  The
 *           epilogue undoes both scales exactly (powers of two).
 *   FP16    the scaled hi*hi product alone (one fp16 product, about 2^-11
 *           relative per operand): the fast low-precision form.
 *
 * 1. k_row_scan / k_col_scan: per row of A and column of B, the largest
 *    magnitude of each channel and whether any colour is non-zero.
 *    k_compact: the lists of non-zero rows and columns and their scale
 *    exponents.  k_zero_fill: the outputs of zero rows and columns.
 * 2. k_split_a / k_split_b (memory bound) gather the non-zero rows and
 *    columns, scale them, and split them into 16-bit hi/lo planes, K
 *    contiguous, zero padded to the tile sizes: As[c][h][Mp][Kp] and
 *    Bs[c][h][Np][Kp] (B transposed through shared memory).
 * 3. k_dct_tc: a persistent kernel, one CTA per SM, 10 warps:
 *      warp 0  TMA producer: 128x64 (A) and 256x64 (B) 16-bit boxes with the
 *              128-byte swizzle, of each plane in use, into a ring of
 *              shared-memory stages (2 stages of 96 KB for the split forms,
 *              4 of 48 KB for FP16)
 *      warp 1  allocates 512 TMEM columns (two 128x256 FP32 accumulators)
 *              and one lane issues tcgen05.mma (M=128, N=256, K=16),
 *              committing each stage back to the producer and each finished
 *              K chunk (128 of K) to the epilogue
 *      warps 2-9  epilogue: tcgen05.ld of a finished chunk (each warp its
 *              32-lane TMEM sub-partition and one half of the columns) into
 *              FP32 registers.  The FP32 accumulation inside the tensor
 *              cores rounds with a bias: its error grows linearly with the
 *              number of products in one accumulator (measured, with all of
 *              K in one accumulator: mean relative error 3.2e-6 at K = 700,
 *              1.2e-5 at K = 2306; 1.5e-6 with chunks of 256 of K).  Summing
 *              chunks of 128 of K in registers with IEEE rounding bounds
 *              that growth.  The two accumulators
 *              alternate, so the epilogue of one chunk overlaps the products
 *              of the next.  The finished tile is transposed through shared
 *              memory, 32 x 32 per warp, so that each store instruction
 *              writes 32 consecutive columns of one output row.
 *    Tiles run channel-innermost, so the three channels of one output block
 *    are written at the same time by neighbouring CTAs and merge in L2, and
 *    in groups of 16 row tiles for operand reuse in L2.
 *
 * Every wait on an mbarrier is bounded (two seconds of %globaltimer); on
 * expiry the CTA records an error code, stops issuing work, waits (bounded,
 * two seconds) for its copies and products in flight and frees its tensor
 * memory, and the host reports GB_ECUDA.  The environment variable
 * GB_DCT_WAIT_NS, read at each call, shortens the limit of the pipeline's
 * waits (not of the final drains), so that tests can make a wait run out
 * without any copy or product being left in flight.
 */
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "dct.h"
#include "../../include/gbrad.h"

namespace {

constexpr int TM = 128, TN = 256, TK = 64;          /* tile; TK 16-bit elements = 128 bytes */
constexpr int A_BYTES = TM * TK * 2;                /* 16 KB per plane */
constexpr int B_BYTES = TN * TK * 2;                /* 32 KB per plane */
constexpr int TMEM_COLS = 512;                      /* 2 accumulators x TN */
constexpr int GROUP_M = 16;                         /* row tiles per raster group */
constexpr int NTHREADS = 320;                       /* producer, MMA, 8 epilogue warps */
constexpr int CHUNK_KB = 2;                         /* K blocks per accumulator chunk (K = 128) */
constexpr int EPI_COLS = TN / 2;                    /* columns per epilogue thread */
constexpr int XPOSE_BYTES = 8 * 32 * 32 * 4;        /* one 32 x 32 float block per epilogue warp */
constexpr uint64_t WAIT_NS = 2000000000ull;         /* limit of every wait: 2 s */

/* NH planes per operand (2: hi and lo, 1: hi only) */
template <int NH>
struct Ring {
    static constexpr int STAGE_BYTES = NH * (A_BYTES + B_BYTES);
    static constexpr int STAGES = NH == 2 ? 2 : 4;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + XPOSE_BYTES + 1024 /* alignment */ + 256 /* barriers */;
};

/* tcgen05 instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B
 * of one type (bits 7-9, 10-12: 0 F16, 1 BF16), both K-major (bits 15, 16 =
 * 0), N >> 3 at bit 17, M >> 4 at bit 24 */
template <bool BF16>
__host__ __device__ constexpr uint32_t idesc()
{
    return (1u << 4) | (BF16 ? (1u << 7) | (1u << 10) : 0u) | ((uint32_t)(TN >> 3) << 17) |
           ((uint32_t)(TM >> 4) << 24);
}

enum { ERR_NONE = 0, ERR_FULL = 1, ERR_EMPTY = 2, ERR_TFULL = 3, ERR_TEMPTY = 4, ERR_DRAIN = 5 };

struct Shape {
    int M, K, N;          /* true sizes */
    int Mc, Nc;           /* non-zero rows of A, columns of B */
    int Mp, Kp, Np;       /* Mc, K, Nc padded to TM, TK, TN */
    int mt, nt, kb;       /* tile counts, K blocks */
    long long tiles;      /* mt * nt * 3 */
    int scaled;           /* rows and columns carry power-of-two scales */
    unsigned long long wait_ns;
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

/* Wait for the phase of `parity` to complete, at most wait_ns.  With
 * `respect_abort`, give up at once when the CTA has aborted. */
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err, int code,
                          uint64_t wait_ns, bool respect_abort = true)
{
    if (mbar_try(bar, parity))
        return true;
    uint64_t t0 = globaltimer();
    for (;;) {
        if (respect_abort && *abort_flag)
            return false;
        if (mbar_try(bar, parity))
            return true;
        if (globaltimer() - t0 > wait_ns) {
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

template <uint32_t IDESC>
__device__ __forceinline__ void mma16(uint32_t dt, uint64_t a, uint64_t b, uint32_t acc)
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

/* The product over the compacted operands.  rowidx/colidx map compact rows
 * and columns to output rows and columns; ea[c][i] and eb[c][j] are the
 * scale exponents of compact row i and column j (scaled forms). */
template <int NH, bool BF16>
__global__ void __launch_bounds__(NTHREADS, 1)
k_dct_tc(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, Shape s,
         float *__restrict__ C, const int *__restrict__ rowidx, const int *__restrict__ colidx,
         const int *__restrict__ ea, const int *__restrict__ eb, int *err)
{
    using R = Ring<NH>;
    constexpr int STAGES = R::STAGES, STAGE_BYTES = R::STAGE_BYTES;
    constexpr uint32_t IDESC = idesc<BF16>();
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *xpose = (float *)(smem + STAGES * STAGE_BYTES);
    uint64_t *bars = (uint64_t *)(smem + STAGES * STAGE_BYTES + XPOSE_BYTES);
    /* bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], drain */
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES;
    const uint32_t tfull0 = empty0 + 8 * STAGES, tempty0 = tfull0 + 16, drain = tempty0 + 16;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * STAGES + 5);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t wns = s.wait_ns;

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
                const int ya = NH * c * s.Mp + mi * TM, yb = NH * c * s.Np + ni * TN;
                for (int kb = 0; kb < s.kb; kb++, it++) {
                    const int st = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                    if (!mbar_wait(empty0 + 8 * st, ph ^ 1, abort_flag, err, ERR_EMPTY, wns))
                        break;
                    const uint32_t base = smem_u32(smem + st * STAGE_BYTES), fb = full0 + 8 * st;
                    mbar_expect_tx(fb, STAGE_BYTES);
#pragma unroll
                    for (int h = 0; h < NH; h++) {
                        tma_load_2d(base + h * A_BYTES, &mapA, kb * TK, ya + h * s.Mp, fb);
                        tma_load_2d(base + NH * A_BYTES + h * B_BYTES, &mapB, kb * TK, yb + h * s.Np, fb);
                    }
                }
            }
            /* copies in flight land before the CTA can exit */
            for (long long j = it - STAGES; j < it; j++) {
                if (j < 0)
                    continue;
                mbar_wait(full0 + 8 * (int)(j % STAGES), (uint32_t)((j / STAGES) & 1), abort_flag, err, ERR_FULL,
                          WAIT_NS, false);
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
                    if (!mbar_wait(tempty0 + 8 * buf, use ^ 1, abort_flag, err, ERR_TEMPTY, wns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dt = tmem + (uint32_t)(buf * TN);
                    const int k1 = k0 + CHUNK_KB < s.kb ? k0 + CHUNK_KB : s.kb;
                    for (int kb = k0; kb < k1; kb++, it++) {
                        const int st = (int)(it % STAGES);
                        const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                        if (!mbar_wait(full0 + 8 * st, ph, abort_flag, err, ERR_FULL, wns)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t base = smem_u32(smem + st * STAGE_BYTES);
#pragma unroll
                        for (int j = 0; j < TK / 16; j++) {
                            const uint64_t ahi = sdesc(base + 32 * j);
                            const uint64_t bhi = sdesc(base + NH * A_BYTES + 32 * j);
                            mma16<IDESC>(dt, ahi, bhi, (kb != k0) | (j != 0));
                            if (NH == 2) {
                                const uint64_t alo = sdesc(base + A_BYTES + 32 * j);
                                const uint64_t blo = sdesc(base + NH * A_BYTES + B_BYTES + 32 * j);
                                mma16<IDESC>(dt, ahi, blo, 1);
                                mma16<IDESC>(dt, alo, bhi, 1);
                            }
                        }
                        mma_commit(empty0 + 8 * st);      /* stage free once these products finish */
                    }
                    if (ok)
                        mma_commit(tfull0 + 8 * buf);     /* chunk complete */
                }
            }
            /* every product issued has finished before tensor memory is freed */
            mma_commit(drain);
            mbar_wait(drain, 0, abort_flag, err, ERR_DRAIN, WAIT_NS, false);
        }
        __syncwarp();
    } else {
        /* ---------------- epilogue: warps 2..9; TMEM sub-partition warp % 4,
         * column half (warp - 2) / 4.  Each K chunk's FP32 accumulator is
         * added into registers (IEEE round to nearest), so the tensor cores'
         * accumulation rounding acts on chains of CHUNK_KB * TK products only */
        const int sub = warp & 3, half = (warp - 2) >> 2;
        float *xs = xpose + (warp - 2) * 1024;
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
                ok = mbar_wait(tfull0 + 8 * buf, use, abort_flag, err, ERR_TFULL, wns);
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
            /* this warp's 32 compact rows: lane r holds row r's output index
             * and scale exponent, broadcast below */
            const int ir = mi * TM + sub * 32 + lane;
            const int my_m = ir < s.Mc ? rowidx[ir] : -1;
            const int my_ea = (ir < s.Mc && s.scaled) ? ea[(long long)c * s.Mc + ir] : 0;
            const int nrows = min(32, s.Mc - (mi * TM + sub * 32));
            const int jc0 = ni * TN + half * EPI_COLS;
#pragma unroll
            for (int b = 0; b < EPI_COLS / 32; b++) {
                /* lane = row, i = column -> xs[row][i ^ row]: no bank conflicts */
#pragma unroll
                for (int i = 0; i < 32; i++)
                    xs[lane * 32 + (i ^ lane)] = acc[b * 32 + i];
                __syncwarp();
                const int jc = jc0 + b * 32 + lane;       /* this lane's compact column */
                const bool colok = jc < s.Nc;
                const int n = colok ? colidx[jc] : 0;
                const int ebn = (colok && s.scaled) ? eb[(long long)c * s.Nc + jc] : 0;
                for (int r = 0; r < nrows; r++) {
                    const float v = xs[r * 32 + (lane ^ r)];
                    const int m = __shfl_sync(0xffffffffu, my_m, r);
                    const int e = __shfl_sync(0xffffffffu, my_ea, r) + ebn;
                    if (colok)
                        C[((long long)m * s.N + n) * 3 + c] = s.scaled ? ldexpf(v, -e) : v;
                }
                __syncwarp();
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

/* ----------------------------------------------------------------- scans */

/* Per row m of A[m][k][c]: the largest magnitude of each channel (as the
 * bits of a non-negative float, which order as unsigned integers) and
 * whether any byte of the row is non-zero.  One warp per row. */
__global__ void k_row_scan(const float *__restrict__ A, int M, int K, unsigned *__restrict__ rowmax,
                           int *__restrict__ rowflag)
{
    const int m = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (m >= M)
        return;
    const float *a = A + (long long)m * K * 3;
    unsigned mx[3] = {0, 0, 0}, any = 0;
    const int n3 = 3 * K;
    for (int j = lane; j < n3; j += 32) {
        const unsigned u = __float_as_uint(a[j]);
        any |= u;
        const int ch = j % 3;
        const unsigned v = u & 0x7fffffffu;
        mx[ch] = v > mx[ch] ? v : mx[ch];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        any |= __shfl_xor_sync(0xffffffffu, any, o);
#pragma unroll
        for (int ch = 0; ch < 3; ch++)
            mx[ch] = max(mx[ch], __shfl_xor_sync(0xffffffffu, mx[ch], o));
    }
    if (lane == 0) {
        rowflag[m] = any != 0;
        rowmax[3 * m] = mx[0];
        rowmax[3 * m + 1] = mx[1];
        rowmax[3 * m + 2] = mx[2];
    }
}

/* Per column n of B[k][n][c], over the rows k in [blockIdx.y * kspan, ...):
 * the same, merged with atomics (colmax and colflag start at zero). */
__global__ void k_col_scan(const float *__restrict__ B, int K, int N, int kspan, unsigned *__restrict__ colmax,
                           int *__restrict__ colflag)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;   /* n * 3 + c */
    if (j >= 3LL * N)
        return;
    const int k0 = blockIdx.y * kspan, k1 = min(K, k0 + kspan);
    unsigned mx = 0, any = 0;
    for (int k = k0; k < k1; k++) {
        const unsigned u = __float_as_uint(B[(long long)k * N * 3 + j]);
        any |= u;
        mx = max(mx, u & 0x7fffffffu);
    }
    if (mx)
        atomicMax(colmax + j, mx);
    if (any)
        atomicOr(colflag + j / 3, 1);
}

/* The exponent that brings a largest magnitude into [2^14, 2^15). */
__device__ __forceinline__ int scale_exp(unsigned maxbits)
{
    const float mx = __uint_as_float(maxbits);
    if (maxbits == 0 || !isfinite(mx))
        return 0;
    return 14 - ilogbf(mx);
}

/* The list of non-zero entries of flag[0..n) in order (idx, *count) and,
 * with maxv, the scale exponent of each channel of each listed entry
 * (exps[c][i]).  One block of 1024 threads, each a contiguous segment. */
__global__ void __launch_bounds__(1024) k_compact(const int *__restrict__ flag, int n,
                                                  const unsigned *__restrict__ maxv, int *__restrict__ idx,
                                                  int *__restrict__ exps, int *__restrict__ count)
{
    __shared__ int part[1024];
    const int t = threadIdx.x, seg = (n + 1023) / 1024;
    const int b = min(n, t * seg), e = min(n, b + seg);
    int cnt = 0;
    for (int i = b; i < e; i++)
        cnt += flag[i] != 0;
    part[t] = cnt;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {     /* inclusive scan */
        const int v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    const int total = part[1023];
    int pos = part[t] - cnt;
    for (int i = b; i < e; i++)
        if (flag[i]) {
            idx[pos] = i;
            if (maxv) {
                exps[pos] = scale_exp(maxv[3 * i]);
                exps[(long long)total + pos] = scale_exp(maxv[3 * i + 1]);
                exps[2LL * total + pos] = scale_exp(maxv[3 * i + 2]);
            }
            pos++;
        }
    if (t == 0)
        *count = total;
}

/* Outputs of zero rows of A or zero columns of B are zero (the product
 * kernel writes the others): rows over the grid's y, columns over x. */
__global__ void k_zero_fill(float *__restrict__ C, const int *__restrict__ rowflag, const int *__restrict__ colflag,
                            int M, int N)
{
    for (int m = blockIdx.y; m < M; m += gridDim.y) {
        const bool zr = !rowflag[m];
        float *row = C + (long long)m * N * 3;
        for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
            if (zr || !colflag[n]) {
                row[3 * n] = 0.f;
                row[3 * n + 1] = 0.f;
                row[3 * n + 2] = 0.f;
            }
    }
}

/* ----------------------------------------------------------------- splits */

template <bool BF16>
struct Half16;
template <>
struct Half16<true> {
    typedef __nv_bfloat16 T;
    static __device__ __forceinline__ T rn(float x) { return __float2bfloat16_rn(x); }
    static __device__ __forceinline__ float f(T h) { return __bfloat162float(h); }
};
template <>
struct Half16<false> {
    typedef __half T;
    static __device__ __forceinline__ T rn(float x) { return __float2half_rn(x); }
    static __device__ __forceinline__ float f(T h) { return __half2float(h); }
};

/* Compact row i of A (row rowidx[i]), scaled by 2^ea[c][i] -> As[c][h][Mp][Kp]
 * hi (and lo), one thread per element of the padded plane (zeros in the
 * padding). */
template <int NH, bool BF16>
__global__ void k_split_a(const float *__restrict__ A, typename Half16<BF16>::T *__restrict__ As,
                          const int *__restrict__ rowidx, const int *__restrict__ ea, Shape s)
{
    typedef Half16<BF16> H;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)s.Mp * s.Kp)
        return;
    const int r = (int)(i / s.Kp), k = (int)(i % s.Kp);
    const bool in = r < s.Mc && k < s.K;
    const size_t plane = (size_t)s.Mp * s.Kp;
    const float *a = in ? A + 3 * ((long long)rowidx[r] * s.K + k) : A;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float x = in ? a[c] : 0.f;
        if (in && s.scaled)
            x = ldexpf(x, ea[(long long)c * s.Mc + r]);
        const typename H::T hi = H::rn(x);
        As[(NH * c) * plane + i] = hi;
        if (NH == 2)
            As[(NH * c + 1) * plane + i] = H::rn(x - H::f(hi));
    }
}

/* Compact column j of B (column colidx[j]), scaled by 2^eb[c][j] ->
 * Bs[c][h][Np][Kp] (transposed, K contiguous) through a 32x32 shared tile
 * per channel; the grid covers the padded plane */
template <int NH, bool BF16>
__global__ void k_split_b(const float *__restrict__ B, typename Half16<BF16>::T *__restrict__ Bs,
                          const int *__restrict__ colidx, const int *__restrict__ eb, Shape s)
{
    typedef Half16<BF16> H;
    __shared__ float tile[3][32][33];
    const int k0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;          /* 32 x 8 */
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r;
        for (int q = tx; q < 96; q += 32) {
            const int j = j0 + q / 3, c = q % 3;
            float x = 0.f;
            if (k < s.K && j < s.Nc) {
                x = B[((size_t)k * s.N + colidx[j]) * 3 + c];
                if (s.scaled)
                    x = ldexpf(x, eb[(long long)c * s.Nc + j]);
            }
            tile[c][r][q / 3] = x;
        }
    }
    __syncthreads();
    const size_t plane = (size_t)s.Np * s.Kp;
    for (int r = ty; r < 32; r += 8) {            /* padded plane: zeros beyond K, Nc */
        const int j = j0 + r, k = k0 + tx;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float x = tile[c][tx][r];
            const typename H::T hi = H::rn(x);
            Bs[(NH * c) * plane + (size_t)j * s.Kp + k] = hi;
            if (NH == 2)
                Bs[(NH * c + 1) * plane + (size_t)j * s.Kp + k] = H::rn(x - H::f(hi));
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

/* rows x Kp 16-bit matrix, box TK x box_rows, 128-byte swizzle */
bool make_map(CUtensorMap *m, const void *base, uint64_t rows, uint64_t kp, uint32_t box_rows, bool bf16)
{
    auto fn = encode_fn();
    if (!fn)
        return false;
    cuuint64_t dims[2] = {kp, rows};
    cuuint64_t strides[1] = {kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)TK, box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
              const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

/* Work buffers of one device, kept between calls and grown on demand;
 * calls are serialised on them. */
struct Work {
    unsigned char *p = nullptr;
    size_t size = 0;
};

template <int NH, bool BF16>
int run_tc(const float *A, const float *B, Shape s, float *C, cudaStream_t st, unsigned char *ws,
           const size_t *off, int sms, std::string &err)
{
    typedef typename Half16<BF16>::T T;
    int *d_err = (int *)(ws + off[0]);
    int *rowidx = (int *)(ws + off[3]), *colidx = (int *)(ws + off[4]);
    int *ea = (int *)(ws + off[5]), *eb = (int *)(ws + off[6]);
    T *As = (T *)(ws + off[8]), *Bs = (T *)(ws + off[9]);
    const long long na = (long long)s.Mp * s.Kp;
    k_split_a<NH, BF16><<<(unsigned)((na + 255) / 256), 256, 0, st>>>(A, As, rowidx, ea, s);
    k_split_b<NH, BF16><<<dim3((unsigned)(s.Np / 32), (unsigned)(s.Kp / 32)), dim3(32, 8), 0, st>>>(B, Bs, colidx,
                                                                                                 eb, s);
    CUtensorMap ma, mb;
    if (!make_map(&ma, As, (uint64_t)NH * 3 * s.Mp, (uint64_t)s.Kp, TM, BF16) ||
        !make_map(&mb, Bs, (uint64_t)NH * 3 * s.Np, (uint64_t)s.Kp, TN, BF16)) {
        err = "cannot encode the TMA tensor maps";
        return GB_ECUDA;
    }
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_dct_tc<NH, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Ring<NH>::SMEM_BYTES) != cudaSuccess) {
            err = "cannot reserve shared memory for the tensor-core kernel";
            return GB_ECUDA;
        }
        attr_set = true;
    }
    const long long grid = s.tiles < sms ? s.tiles : sms;
    k_dct_tc<NH, BF16><<<(unsigned)grid, NTHREADS, Ring<NH>::SMEM_BYTES, st>>>(ma, mb, s, C, rowidx, colidx, ea,
                                                                              eb, d_err);
    return GB_OK;
}

}  // namespace

int gb_dct_tc(const float *A, const float *B, int64_t M, int64_t K, int64_t N, int mode, float *C, cudaStream_t st,
              std::string &err)
{
    auto rnd = [](int64_t x, int64_t q) { return (x + q - 1) / q * q; };
    if (M > (1 << 24) || K > (1 << 20) || N > (1 << 24) || M * K > (1ll << 37) || K * N > (1ll << 37)) {
        err = "matrix too large for the tensor-core path";
        return GB_EINVAL;
    }
    const int NH = mode == GB_DCT_FP16 ? 1 : 2;
    const bool scaled = mode != GB_DCT_BF16X3;
    const int64_t Mp_max = rnd(M, TM), Np_max = rnd(N, TN), Kp = rnd(K, TK);
    /* workspace layout: [0] error flag + counts, [1] row max, [2] column
     * max, [3] row list, [4] column list, [5] row exponents, [6] column
     * exponents, [7] row and column flags, [8] A planes, [9] B planes */
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t off[11];
    off[0] = 0;
    off[1] = 256;
    off[2] = off[1] + up((size_t)M * 3 * 4);
    off[3] = off[2] + up((size_t)N * 3 * 4);
    off[4] = off[3] + up((size_t)M * 4);
    off[5] = off[4] + up((size_t)N * 4);
    off[6] = off[5] + up((size_t)M * 3 * 4);
    off[7] = off[6] + up((size_t)N * 3 * 4);
    off[8] = off[7] + up((size_t)(M + N) * 4);
    off[9] = off[8] + up((size_t)NH * 3 * Mp_max * Kp * 2);
    off[10] = off[9] + up((size_t)NH * 3 * Np_max * Kp * 2);
    const size_t total = off[10];
    static std::mutex lock;
    static Work work[64];
    static int sms_of[64];
    std::lock_guard<std::mutex> guard(lock);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        err = "no usable CUDA device";
        return GB_ECUDA;
    }
    Work &w = work[dev];
    if (w.size < total) {
        if (w.p) {
            cudaStreamSynchronize(st);
            cudaFree(w.p);
        }
        w.p = nullptr;
        w.size = 0;
        if (cudaMalloc(&w.p, total) != cudaSuccess) {
            cudaGetLastError();
            w.p = nullptr;
            err = "cannot allocate the tensor-core operand planes";
            return GB_ENOMEM;
        }
        w.size = total;
    }
    if (!sms_of[dev])
        cudaDeviceGetAttribute(&sms_of[dev], cudaDevAttrMultiProcessorCount, dev);
    unsigned char *ws = w.p;
    int *d_err = (int *)ws, *d_cnt = d_err + 1;
    unsigned *rowmax = (unsigned *)(ws + off[1]), *colmax = (unsigned *)(ws + off[2]);
    int *rowidx = (int *)(ws + off[3]), *colidx = (int *)(ws + off[4]);
    int *ea = (int *)(ws + off[5]), *eb = (int *)(ws + off[6]);
    int *rowflag = (int *)(ws + off[7]), *colflag = rowflag + M;

    auto cuda_fail = [&](const char *what) {
        err = std::string(what) + ": " + cudaGetErrorString(cudaGetLastError());
        cudaStreamSynchronize(st);
        return GB_ECUDA;
    };
    /* zero rows and columns, scales, and the lists of the others */
    if (cudaMemsetAsync(ws, 0, 256, st) != cudaSuccess ||
        cudaMemsetAsync(colmax, 0, (size_t)N * 3 * 4, st) != cudaSuccess ||
        cudaMemsetAsync(colflag, 0, (size_t)N * 4, st) != cudaSuccess)
        return cuda_fail("memset");
    k_row_scan<<<(unsigned)((M * 32LL + 255) / 256), 256, 0, st>>>(A, (int)M, (int)K, rowmax, rowflag);
    const int kspan = 64;
    k_col_scan<<<dim3((unsigned)((3 * N + 255) / 256), (unsigned)((K + kspan - 1) / kspan)), 256, 0, st>>>(
        B, (int)K, (int)N, kspan, colmax, colflag);
    k_compact<<<1, 1024, 0, st>>>(rowflag, (int)M, scaled ? rowmax : nullptr, rowidx, ea, d_cnt);
    k_compact<<<1, 1024, 0, st>>>(colflag, (int)N, scaled ? colmax : nullptr, colidx, eb, d_cnt + 1);
    {
        const int gx = (int)std::min<int64_t>((N + 255) / 256, 64);
        const int gy = (int)std::min<int64_t>(M, std::max(1, 8 * sms_of[dev] / gx));
        k_zero_fill<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, st>>>(C, rowflag, colflag, (int)M, (int)N);
    }
    int cnt[2] = {0, 0};
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(cnt, d_cnt, sizeof cnt, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return cuda_fail("scan of zero rows and columns");
    if (cnt[0] == 0 || cnt[1] == 0)
        return GB_OK;

    Shape s;
    s.M = (int)M;
    s.K = (int)K;
    s.N = (int)N;
    s.Mc = cnt[0];
    s.Nc = cnt[1];
    s.Mp = (int)rnd(s.Mc, TM);
    s.Kp = (int)Kp;
    s.Np = (int)rnd(s.Nc, TN);
    s.mt = s.Mp / TM;
    s.nt = s.Np / TN;
    s.kb = s.Kp / TK;
    s.tiles = (long long)s.mt * s.nt * 3;
    s.scaled = scaled;
    s.wait_ns = WAIT_NS;
    if (const char *w = getenv("GB_DCT_WAIT_NS")) {
        const unsigned long long v = strtoull(w, nullptr, 10);
        if (v > 0 && v < WAIT_NS)
            s.wait_ns = v;
    }
    int rc;
    if (mode == GB_DCT_BF16X3)
        rc = run_tc<2, true>(A, B, s, C, st, ws, off, sms_of[dev], err);
    else if (mode == GB_DCT_FP16X3)
        rc = run_tc<2, false>(A, B, s, C, st, ws, off, sms_of[dev], err);
    else
        rc = run_tc<1, false>(A, B, s, C, st, ws, off, sms_of[dev], err);
    if (rc < 0) {
        cudaStreamSynchronize(st);
        return rc;
    }
    if (cudaGetLastError() != cudaSuccess)
        return cuda_fail("tensor-core launch");
    int h_err = 0;
    if (cudaMemcpyAsync(&h_err, d_err, sizeof h_err, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return cuda_fail("tensor-core product");
    if (h_err) {
        err = "tensor-core pipeline wait expired (code " + std::to_string(h_err) + ")";
        return GB_ECUDA;
    }
    return GB_OK;
}
