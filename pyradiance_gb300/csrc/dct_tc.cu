/*
 * dct_tc.cu -- dctimestep's product on the 5th-generation tensor cores.
 *
 * R[m,n,c] = sum_k A[m,k,c] * B[k,n,c] for each colour channel c
 * (util/cmatrix.c:421-474 cm_multiply; the channels do not mix), with the
 * reference's skip of all-zero columns of B (a column is zero when every
 * byte of its colours is, cmatrix.c:435-450): their outputs are written as
 * zeros and the product runs over the other columns only.  All-zero rows of
 * A (rare in daylight coefficients) are not skipped: their products are
 * exact zeros, the same output.  Three arithmetic forms share one kernel:
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
 *           relative per operand): the fast low-precision form, with all
 *           of K accumulated in the tensor cores.
 *
 * 1. k_col_scan: per column of B, the largest magnitude of each channel
 *    and whether any colour is non-zero; k_compact: the list of non-zero
 *    columns and their scale exponents (the one host synchronisation of a
 *    call reads their count).
 * 2. k_split_rows (memory bound, one pass over A from HBM): per row of A,
 *    its scale exponents, then the row scaled and split into 16-bit hi/lo
 *    planes.  k_split_b gathers, scales and splits the non-zero columns of
 *    B.  Both K contiguous, zero padded to the tile sizes: As[c][h][Mp][Kp]
 *    and Bs[c][h][Np][Kp] (B transposed through shared memory).
 * 3. k_dct_tc: a persistent kernel, one CTA per SM, 12 warps:
 *      warp 0  TMA producer: 128x32 (A) and 256x32 (B) 16-bit boxes with the
 *              64-byte swizzle, of each plane in use, into a ring of
 *              shared-memory stages (4 stages of 48 KB for the split forms,
 *              8 of 24 KB for FP16): three stages in flight while the
 *              products run on the fourth.  (Two stages of 96 KB, with
 *              128-byte boxes, left the products waiting on the copies.)
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
 *      warps 10-11  the zeros of the zero columns of B among each unit's
 *              output columns (from its first column to the next column
 *              tile's first), all three channels of a third of the rows
 *              per channel unit, as runs of float4s (single floats at run
 *              ends), each unit's while its products run (paced by the MMA
 *              issuer's unit count); every output is written once, by this
 *              kernel.  (Unpaced, the float4 stores of the first units
 *              competed with their copies: FP16X3 9% slower.)
 *    Units run channel-innermost, so the three channels of one output block
 *    are written at the same time by neighbouring CTAs and merge in L2, and
 *    in groups of 2048 rows of A for operand reuse in L2.
 *    With two or more row tiles the CTAs run in clusters of two on row
 *    tiles 2p and 2p + 1 of the same column tile: each copies its A tile
 *    and one half of the B tile, multicast to both CTAs (half the L2 reads
 *    of B), and a stage is released when both CTAs' products over it are
 *    done.
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

constexpr int TM = 128, TN = 256, TK = 32;          /* tile; TK 16-bit elements = 64 bytes */
constexpr int SWZ = TK * 2;                         /* swizzle span: one K row of a box (64 bytes) */
constexpr int A_BYTES = TM * TK * 2;                /* 8 KB per plane */
constexpr int B_BYTES = TN * TK * 2;                /* 16 KB per plane */
constexpr int TMEM_COLS = 512;                      /* 2 accumulators x TN */
constexpr int GROUP_ROWS = 2048;                    /* rows of A per raster group (their planes stay in L2) */
constexpr int NTHREADS = 384;                       /* producer, MMA, 8 epilogue warps, 2 zero-column warps */
constexpr int CHUNK_KB = 128 / TK;                  /* K blocks per accumulator chunk (K = 128) */
/* the FP16 form (one product, operands rounded to 2^-11) accumulates all of
 * K in one accumulator: the tensor cores' accumulation error (about 1e-5)
 * is far below its operand rounding, and the epilogue runs once per tile */
template <int NH>
__host__ __device__ constexpr int chunk_kb() { return NH == 2 ? CHUNK_KB : 1 << 20; }
constexpr int EPI_COLS = TN / 2;                    /* columns per epilogue thread */
constexpr int XPOSE_BYTES = 8 * 32 * 32 * 4;        /* one 32 x 32 float block per epilogue warp */
constexpr uint64_t WAIT_NS = 2000000000ull;         /* limit of every wait: 2 s */

/* NH planes per operand (2: hi and lo, 1: hi only) */
template <int NH>
struct Ring {
    static constexpr int STAGE_BYTES = NH * (A_BYTES + B_BYTES);
    static constexpr int STAGES = NH == 2 ? 4 : 8;
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
    int Nc;               /* non-zero columns of B */
    int Mp, Kp, Np;       /* M, K, Nc padded to the tiles (M to pairs of row tiles in clusters) */
    int mt, nt, kb;       /* tile counts, K blocks */
    long long tiles;      /* mt * nt * 3 */
    int mu;               /* row units: row tiles, or pairs of them in clusters of two */
    long long units;      /* mu * nt * 3 */
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

/* the same box into this CTA's and its cluster peer's shared memory (same
 * offset in each), each CTA's mbarrier at the same offset signalled */
__device__ __forceinline__ void tma_load_2d_mc(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar,
                                               uint16_t mask)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster "
        "[%0], [%1, {%2, %3}], [%4], %5;"
        ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar), "h"(mask)
        : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

/* shared-memory matrix descriptor: K-major, rows of SWZ bytes with the
 * SWZ-byte swizzle (layout type 2: 128 bytes, 4: 64 bytes), 8-row groups
 * 8 * SWZ bytes apart (stride byte offset), descriptor version 1 (bit 46) */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    static_assert(SWZ == 128 || SWZ == 64, "swizzle span");
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)((8u * SWZ) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)(SWZ == 128 ? 2 : 4) << 61;
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

/* arrive, once these products finish, on the mbarrier at this offset in
 * every CTA of the mask */
__device__ __forceinline__ void mma_commit_mc(uint32_t bar, uint16_t mask)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;"
                 ::"r"(bar), "h"(mask)
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

/* work unit t -> (channel, row unit, column tile): channel innermost, then
 * the row units of a group of GROUP_ROWS rows (row tiles, or pairs of them)
 * sweeping the column tiles, so that the group's A planes (2048 rows: 57 MB
 * in the split forms) are reused from L2 by every column tile of B.
 * Measured at 16384 x 2306 x 8760: groups of 1024 and 2048 rows take the
 * same time, groups of 4096 rows 4.5% longer. */
template <int CL>
__device__ __forceinline__ void tile_coords(const Shape &s, long long t, int &c, int &mi, int &ni)
{
    constexpr int G = GROUP_ROWS / (TM * CL);
    c = (int)(t % 3);
    const long long u = t / 3;
    const long long per_group = (long long)G * s.nt;
    const int g = (int)(u / per_group);
    const int r = (int)(u % per_group);
    int gm = s.mu - g * G;
    if (gm > G)
        gm = G;
    mi = g * G + r % gm;
    ni = r / gm;
}

/* The product over the rows of A and the compacted columns of B.  colidx
 * maps compact columns to output columns, colflag marks the non-zero
 * columns of B; ea[c][m] and eb[c][j] are the scale exponents of row m and
 * compact column j (scaled forms).  Each tile also writes the zeros of the
 * zero columns among its output columns. */
template <int NH, bool BF16, int CL>
__global__ void __launch_bounds__(NTHREADS, 1)
k_dct_tc(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, Shape s,
         float *__restrict__ C, const int *__restrict__ colidx, const int *__restrict__ colflag,
         const int *__restrict__ ea, const int *__restrict__ eb, int *err)
{
    /* CL = 2: the two CTAs of a cluster take row tiles 2p and 2p + 1 of the
     * same column tile and channel; each loads its own A tile and one half
     * of the shared B tile, multicast into both CTAs, and a stage is free
     * once both CTAs' products over it have finished.  The work units are
     * the pairs of row tiles (s.mu of them), in the same order on both
     * CTAs. */
    const int rank = CL == 2 ? (int)cluster_rank() : 0;
    const int unit0 = blockIdx.x / CL, ustride = gridDim.x / CL;
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
    volatile int *unit_clock = (volatile int *)(tmem_slot + 2);   /* units whose products have begun */
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t wns = s.wait_ns;

    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; i++) {
            mbar_init(full0 + 8 * i, 1);
            mbar_init(empty0 + 8 * i, CL);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(tfull0 + 8 * i, 1);
            mbar_init(tempty0 + 8 * i, 8);           /* one arrival per epilogue warp */
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        *unit_clock = 0;
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
    if (CL == 2)
        cluster_sync_all();              /* the peer's barriers are initialised */
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        /* ---------------- TMA producer */
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapA) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapB) : "memory");
            long long it = 0;
            for (long long t = unit0; t < s.units && !*abort_flag; t += ustride) {
                int c, mi, ni;
                tile_coords<CL>(s, t, c, mi, ni);
                mi = mi * CL + rank;
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
                        if (CL == 2)             /* this CTA's half of the B tile, into both CTAs */
                            tma_load_2d_mc(base + NH * A_BYTES + h * B_BYTES + rank * (B_BYTES / 2), &mapB, kb * TK,
                                           yb + h * s.Np + rank * (TN / 2), fb, (uint16_t)3);
                        else
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
            int nunit = 0;
            for (long long t = unit0; t < s.units && ok; t += ustride) {
                *unit_clock = ++nunit;           /* paces the zero-column warps */
                for (int k0 = 0; k0 < s.kb && ok; k0 += chunk_kb<NH>(), cl++) {
                    const int buf = (int)(cl & 1);
                    const uint32_t use = (uint32_t)((cl >> 1) & 1);
                    if (!mbar_wait(tempty0 + 8 * buf, use ^ 1, abort_flag, err, ERR_TEMPTY, wns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dt = tmem + (uint32_t)(buf * TN);
                    const int k1 = k0 + chunk_kb<NH>() < s.kb ? k0 + chunk_kb<NH>() : s.kb;
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
                        if (CL == 2)                      /* the stage is free in both CTAs once */
                            mma_commit_mc(empty0 + 8 * st, (uint16_t)3);   /* both CTAs' products finish */
                        else
                            mma_commit(empty0 + 8 * st);  /* stage free once these products finish */
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
    } else if (warp < 10) {
        /* ---------------- epilogue: warps 2..9; TMEM sub-partition warp % 4,
         * column half (warp - 2) / 4.  Each K chunk's FP32 accumulator is
         * added into registers (IEEE round to nearest), so the tensor cores'
         * accumulation rounding acts on chains of CHUNK_KB * TK products only
         * (split forms) */
        const int sub = warp & 3, half = (warp - 2) >> 2;
        float *xs = xpose + (warp - 2) * 1024;
        long long cl = 0;
        bool ok = true;
        for (long long t = unit0; t < s.units && ok; t += ustride) {
            /* the tile's rows, columns and scale exponents, loaded now so
             * that their latency hides behind the products */
            int c, mi, ni;
            tile_coords<CL>(s, t, c, mi, ni);
            mi = mi * CL + rank;
            const int row0 = mi * TM + sub * 32, ir = row0 + lane;
            const int my_ea = (ir < s.M && s.scaled) ? ea[(long long)c * s.M + ir] : 0;
            const int nrows = min(32, s.M - row0);
            const int jc0 = ni * TN + half * EPI_COLS;
            int ncol[EPI_COLS / 32], ecol[EPI_COLS / 32];   /* per block: this lane's column, its exponent */
#pragma unroll
            for (int b = 0; b < EPI_COLS / 32; b++) {
                const int jc = jc0 + b * 32 + lane;
                ncol[b] = jc < s.Nc ? colidx[jc] : -1;
                ecol[b] = (jc < s.Nc && s.scaled) ? eb[(long long)c * s.Nc + jc] : 0;
            }
            float acc[EPI_COLS];
#pragma unroll
            for (int i = 0; i < EPI_COLS; i++)
                acc[i] = 0.f;
            for (int k0 = 0; k0 < s.kb; k0 += chunk_kb<NH>(), cl++) {
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
                __syncwarp();
                if (lane == 0)
                    mbar_arrive(tempty0 + 8 * buf);
            }
            if (!ok)
                break;
            /* this warp's 32 rows: lane r holds row r's scale exponent,
             * broadcast below */
#pragma unroll
            for (int b = 0; b < EPI_COLS / 32; b++) {
                /* lane = row, i = column -> xs[row][i ^ row]: no bank conflicts */
#pragma unroll
                for (int i = 0; i < 32; i++)
                    xs[lane * 32 + (i ^ lane)] = acc[b * 32 + i];
                __syncwarp();
                const bool colok = ncol[b] >= 0;         /* this lane's compact column exists */
                const int n = colok ? ncol[b] : 0;
                const int ebn = ecol[b];
                float *out = C + ((long long)row0 * s.N + n) * 3 + c;
                const long long rstride = 3LL * s.N;
                for (int r = 0; r < nrows; r++, out += rstride) {
                    const float v = xs[r * 32 + (lane ^ r)];
                    const int e = __shfl_sync(0xffffffffu, my_ea, r) + ebn;
                    /* v * 2^-e: one multiply by the power of two when it is a
                     * normal float (exact, or rounded once as ldexpf rounds) */
                    if (colok)
                        *out = !s.scaled                  ? v
                               : (e >= -126 && e <= 126) ? v * __int_as_float((127 - e) << 23)
                                                         : ldexpf(v, -e);
                }
                __syncwarp();
            }
        }
    } else {
        /* ---------------- warps 10-11: the outputs of the zero columns of
         * B.  For each unit of this CTA, among the unit's output columns
         * (from its first column to the next column tile's first; from 0
         * for the first tile, to N for the last), all three channels, in
         * the unit's rows r with r % 3 == c (the unit's channel): runs of
         * consecutive floats, written while the products run.  The three
         * channel units of a tile cover all its rows. */
        const int hw = warp - 10;
        const long long rstride = 3LL * s.N;
        const bool vec4 = (s.N & 3) == 0 && ((uintptr_t)C & 15) == 0;
        int nunit = 0;
        for (long long t = unit0; t < s.units && !*abort_flag; t += ustride) {
            /* a unit's zeros while its products run: their stores spread
             * over the kernel instead of competing with the first units'
             * copies (bounded wait; the abort flag ends it too) */
            ++nunit;
            if (*unit_clock < nunit) {
                const uint64_t t0 = globaltimer();
                while (*unit_clock < nunit && !*abort_flag && globaltimer() - t0 < WAIT_NS)
                    __nanosleep(2000);
            }
            int c, mi, ni;
            tile_coords<CL>(s, t, c, mi, ni);
            mi = mi * CL + rank;
            const int lo = ni == 0 ? 0 : colidx[ni * TN];
            const int hi = ni + 1 == s.nt ? s.N : colidx[(ni + 1) * TN];
            const int r1 = min(mi * TM + TM, s.M);
            if (vec4) {
                /* rows 16-byte aligned: windows of 16 steps of 32 float4s;
                 * each lane gathers the 4 bits of its float4 per step once
                 * (the zero pattern is the same in every row), then stores
                 * whole float4s of zeros, and single floats at run ends */
                const int f0 = (3 * lo) & ~3, f1 = 3 * hi;
                for (int w0 = f0; w0 < f1; w0 += 16 * 128) {
                    unsigned long long zmask = 0;
                    for (int i = 0; i < 16 && w0 + 128 * i < f1; i++)
                        for (int q = 0; q < 4; q++) {
                            const int f = w0 + 128 * i + 4 * lane + q;
                            if (f >= 3 * lo && f < f1 && !colflag[f / 3])
                                zmask |= 1ull << (4 * i + q);
                        }
                    unsigned steps = 0;                  /* steps where some lane has zeros */
                    for (int i = 0; i < 16; i++)
                        if (__any_sync(0xffffffffu, ((zmask >> (4 * i)) & 15) != 0))
                            steps |= 1u << i;
                    if (!steps)
                        continue;
                    for (int row = mi * TM + c + 3 * hw; row < r1; row += 6) {
                        float *out = C + row * rstride + w0 + 4 * lane;
                        for (unsigned m = steps; m; m &= m - 1) {
                            const int i = __ffs(m) - 1;
                            const unsigned nib = (unsigned)(zmask >> (4 * i)) & 15u;
                            float *o = out + 128 * i;
                            if (nib == 15u)
                                *reinterpret_cast<float4 *>(o) = make_float4(0.f, 0.f, 0.f, 0.f);
                            else
                                for (unsigned b = nib; b; b &= b - 1)
                                    o[__ffs(b) - 1] = 0.f;
                        }
                    }
                }
                continue;
            }
            /* otherwise windows of 64 x 32 floats, a bit per lane and
             * 32-float step, gathered once, then single-float stores */
            for (int w0 = 3 * lo; w0 < 3 * hi; w0 += 64 * 32) {
                const int w1 = min(3 * hi, w0 + 64 * 32);
                unsigned long long zmask = 0;
                for (int i = 0; w0 + 32 * i < w1; i++) {
                    const int f = w0 + 32 * i + lane;
                    if (f < w1 && !colflag[f / 3])
                        zmask |= 1ull << i;
                }
                if (!__any_sync(0xffffffffu, zmask != 0))
                    continue;
                for (int row = mi * TM + c + 3 * hw; row < r1; row += 6) {
                    float *out = C + row * rstride + w0 + lane;
                    for (unsigned long long m = zmask; m; m &= m - 1)
                        out[32 * __ffsll((long long)m) - 32] = 0.f;
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
    if (CL == 2)
        cluster_sync_all();              /* no copy or arrival of the peer targets this CTA any more */
}

/* ----------------------------------------------------------------- scans */

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

/* ----------------------------------------------------------------- splits */

template <bool BF16>
struct Half16;
template <>
struct Half16<true> {
    typedef __nv_bfloat16 T;
    static __device__ __forceinline__ T rn(float x) { return __float2bfloat16_rn(x); }
    static __device__ __forceinline__ float f(T h) { return __bfloat162float(h); }
    static __device__ __forceinline__ unsigned bits(T h) { return __bfloat16_as_ushort(h); }
};
template <>
struct Half16<false> {
    typedef __half T;
    static __device__ __forceinline__ T rn(float x) { return __float2half_rn(x); }
    static __device__ __forceinline__ float f(T h) { return __half2float(h); }
    static __device__ __forceinline__ unsigned bits(T h) { return __half_as_ushort(h); }
};

/* Row m of A, one block of 256 threads per row of the padded planes: the
 * largest magnitude of each channel gives the row's scale exponents
 * ea[c][m] (scaled forms), and the row, scaled, is split into the hi (and
 * lo) planes As[c][h][Mp][Kp], K contiguous, zeros in the padding (k >= K,
 * m >= M).  The second pass over the row reads it from L2. */
template <int NH, bool BF16>
__global__ void __launch_bounds__(256) k_split_rows(const float *__restrict__ A,
                                                    typename Half16<BF16>::T *__restrict__ As,
                                                    int *__restrict__ ea, Shape s)
{
    typedef Half16<BF16> H;
    __shared__ unsigned red[3][8];
    const int m = blockIdx.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const size_t plane = (size_t)s.Mp * s.Kp;
    const bool live = m < s.M;
    const float *a = A + (size_t)(live ? m : 0) * s.K * 3;
    int e[3] = {0, 0, 0};
    if (live && s.scaled) {
        unsigned mx[3] = {0, 0, 0};
        for (int k = t; k < s.K; k += 256) {
#pragma unroll
            for (int c = 0; c < 3; c++)
                mx[c] = max(mx[c], __float_as_uint(a[3 * k + c]) & 0x7fffffffu);
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            mx[c] = __reduce_max_sync(0xffffffffu, mx[c]);
            if (lane == 0)
                red[c][w] = mx[c];
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 3; c++) {
            unsigned v = 0;
            for (int i = 0; i < 8; i++)
                v = max(v, red[c][i]);
            e[c] = scale_exp(v);
        }
        if (t < 3)
            ea[(long long)t * s.M + m] = e[t];
    }
    unsigned *dst = (unsigned *)(As + (size_t)m * s.Kp);      /* pairs of 16-bit elements */
    for (int k = 2 * t; k < s.Kp; k += 512) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float x0 = live && k < s.K ? a[3 * k + c] : 0.f;
            float x1 = live && k + 1 < s.K ? a[3 * k + 3 + c] : 0.f;
            if (s.scaled) {
                x0 = ldexpf(x0, e[c]);
                x1 = ldexpf(x1, e[c]);
            }
            const typename H::T h0 = H::rn(x0), h1 = H::rn(x1);
            dst[(NH * c) * plane / 2 + k / 2] = H::bits(h0) | (H::bits(h1) << 16);
            if (NH == 2)
                dst[(NH * c + 1) * plane / 2 + k / 2] =
                    H::bits(H::rn(x0 - H::f(h0))) | (H::bits(H::rn(x1 - H::f(h1))) << 16);
        }
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

/* rows x Kp 16-bit matrix, box TK x box_rows, SWZ-byte swizzle */
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
              SWZ == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

/* Work buffers of one device, kept between calls and grown on demand;
 * calls are serialised on them. */
struct Work {
    unsigned char *p = nullptr;
    size_t size = 0;
};

template <int NH, bool BF16, int CL>
int launch_tc(const CUtensorMap &ma, const CUtensorMap &mb, const Shape &s, float *C, cudaStream_t st,
              const int *colidx, const int *colflag, const int *ea, const int *eb, int *d_err, int sms,
              std::string &err)
{
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_dct_tc<NH, BF16, CL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 Ring<NH>::SMEM_BYTES) != cudaSuccess) {
            err = "cannot reserve shared memory for the tensor-core kernel";
            return GB_ECUDA;
        }
        attr_set = true;
    }
    const long long units = s.units;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    cfg.blockDim = dim3(NTHREADS);
    cfg.dynamicSmemBytes = Ring<NH>::SMEM_BYTES;
    cfg.stream = st;
    long long groups = sms / CL;               /* persistent: one CTA per SM */
    if (CL == 2) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cfg.gridDim = dim3((unsigned)(2 * groups));
        int active = 0;                        /* clusters the GPCs hold at once */
        if (cudaOccupancyMaxActiveClusters(&active, k_dct_tc<NH, BF16, CL>, &cfg) == cudaSuccess && active > 0)
            groups = std::min<long long>(groups, active);
        cudaGetLastError();
    }
    groups = std::min<long long>(groups, units);
    cfg.gridDim = dim3((unsigned)(CL * groups));
    if (cudaLaunchKernelEx(&cfg, k_dct_tc<NH, BF16, CL>, ma, mb, s, C, colidx, colflag, ea, eb, d_err) !=
        cudaSuccess) {
        err = std::string("tensor-core launch: ") + cudaGetErrorString(cudaGetLastError());
        return GB_ECUDA;
    }
    return GB_OK;
}

template <int NH, bool BF16>
int run_tc(const float *A, const float *B, Shape s, int cl, float *C, cudaStream_t st, unsigned char *ws,
           const size_t *off, int sms, std::string &err)
{
    typedef typename Half16<BF16>::T T;
    int *d_err = (int *)(ws + off[0]);
    int *colidx = (int *)(ws + off[2]), *colflag = (int *)(ws + off[5]);
    int *ea = (int *)(ws + off[3]), *eb = (int *)(ws + off[4]);
    T *As = (T *)(ws + off[6]), *Bs = (T *)(ws + off[7]);
    k_split_rows<NH, BF16><<<(unsigned)s.Mp, 256, 0, st>>>(A, As, ea, s);
    k_split_b<NH, BF16><<<dim3((unsigned)(s.Np / 32), (unsigned)(s.Kp / 32)), dim3(32, 8), 0, st>>>(B, Bs, colidx,
                                                                                                 eb, s);
    /* with clusters of two each CTA copies one half (TN / 2 rows) of a B tile */
    CUtensorMap ma, mb;
    if (!make_map(&ma, As, (uint64_t)NH * 3 * s.Mp, (uint64_t)s.Kp, TM, BF16) ||
        !make_map(&mb, Bs, (uint64_t)NH * 3 * s.Np, (uint64_t)s.Kp, cl == 2 ? TN / 2 : TN, BF16)) {
        err = "cannot encode the TMA tensor maps";
        return GB_ECUDA;
    }
    if (cl == 2)
        return launch_tc<NH, BF16, 2>(ma, mb, s, C, st, colidx, colflag, ea, eb, d_err, sms, err);
    return launch_tc<NH, BF16, 1>(ma, mb, s, C, st, colidx, colflag, ea, eb, d_err, sms, err);
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
    const int64_t Mp_max = rnd(M, 2 * TM), Np_max = rnd(N, TN), Kp = rnd(K, TK);
    /* workspace layout: [0] error flag + column count, [1] column max, [2]
     * column list, [3] row exponents, [4] column exponents, [5] column
     * flags, [6] A planes, [7] B planes */
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    size_t off[9];
    off[0] = 0;
    off[1] = 256;
    off[2] = off[1] + up((size_t)N * 3 * 4);
    off[3] = off[2] + up((size_t)N * 4);
    off[4] = off[3] + up((size_t)M * 3 * 4);
    off[5] = off[4] + up((size_t)N * 3 * 4);
    off[6] = off[5] + up((size_t)N * 4);
    off[7] = off[6] + up((size_t)NH * 3 * Mp_max * Kp * 2);
    off[8] = off[7] + up((size_t)NH * 3 * Np_max * Kp * 2);
    const size_t total = off[8];
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
    unsigned *colmax = (unsigned *)(ws + off[1]);
    int *colidx = (int *)(ws + off[2]), *eb = (int *)(ws + off[4]), *colflag = (int *)(ws + off[5]);

    auto cuda_fail = [&](const char *what) {
        err = std::string(what) + ": " + cudaGetErrorString(cudaGetLastError());
        cudaStreamSynchronize(st);
        return GB_ECUDA;
    };
    /* zero columns of B, column scales, and the list of the others; rows of
     * A are not compacted (a zero row's products are zeros) */
    if (cudaMemsetAsync(ws, 0, 256, st) != cudaSuccess ||
        cudaMemsetAsync(colmax, 0, (size_t)N * 3 * 4, st) != cudaSuccess ||
        cudaMemsetAsync(colflag, 0, (size_t)N * 4, st) != cudaSuccess)
        return cuda_fail("memset");
    const int kspan = 64;
    k_col_scan<<<dim3((unsigned)((3 * N + 255) / 256), (unsigned)((K + kspan - 1) / kspan)), 256, 0, st>>>(
        B, (int)K, (int)N, kspan, colmax, colflag);
    k_compact<<<1, 1024, 0, st>>>(colflag, (int)N, scaled ? colmax : nullptr, colidx, eb, d_cnt);
    int nc = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&nc, d_cnt, sizeof nc, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return cuda_fail("scan of zero columns");
    if (nc == 0) {                             /* every column of B is zero */
        if (cudaMemsetAsync(C, 0, (size_t)M * N * 3 * 4, st) != cudaSuccess)
            return cuda_fail("memset");
        return GB_OK;
    }

    Shape s;
    s.M = (int)M;
    s.K = (int)K;
    s.N = (int)N;
    s.Nc = nc;
    /* two row tiles share each B tile in clusters of two CTAs (rows padded
     * to a pair of tiles); a single row tile runs alone */
    int cl = rnd(M, TM) >= 2 * TM ? 2 : 1;
    if (const char *e = getenv("GB_DCT_CLUSTER"))
        if (atoi(e) == 1)
            cl = 1;
    s.Mp = (int)rnd(M, cl * TM);
    s.Kp = (int)Kp;
    s.Np = (int)rnd(s.Nc, TN);
    s.mt = s.Mp / TM;
    s.nt = s.Np / TN;
    s.kb = s.Kp / TK;
    s.tiles = (long long)s.mt * s.nt * 3;
    s.mu = s.mt / cl;
    s.units = (long long)s.mu * s.nt * 3;
    s.scaled = scaled;
    s.wait_ns = WAIT_NS;
    if (const char *w = getenv("GB_DCT_WAIT_NS")) {
        const unsigned long long v = strtoull(w, nullptr, 10);
        if (v > 0 && v < WAIT_NS)
            s.wait_ns = v;
    }
    int rc;
    if (mode == GB_DCT_BF16X3)
        rc = run_tc<2, true>(A, B, s, cl, C, st, ws, off, sms_of[dev], err);
    else if (mode == GB_DCT_FP16X3)
        rc = run_tc<2, false>(A, B, s, cl, C, st, ws, off, sms_of[dev], err);
    else
        rc = run_tc<1, false>(A, B, s, cl, C, st, ws, off, sms_of[dev], err);
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
