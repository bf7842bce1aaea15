/*
 * dct.cu -- dctimestep's DC x sky product on CUDA cores.
 *
 * The reference (util/cmatrix.c:421-474, cm_multiply) computes each output
 * element as three independent channel sums accumulated in double over
 * interleaved RGB matrices, skipping all-zero rows and columns.  Here one
 * thread block computes a 64 x 64 output tile for all three channels: the
 * interleaved A and B tiles are staged through shared memory de-interleaved
 * by channel, and each thread accumulates a 4 x 4 x 3 register tile.  The
 * FP32 kernel accumulates in float (the plain baseline); the FP64 kernel
 * accumulates in double like the reference.
 */
#include "dct.h"
#include "../../include/gbrad.h"

#define TM 64
#define TN 64
#define TK 16

template <typename Acc>
__global__ void __launch_bounds__(256) k_dct_simt(const float *__restrict__ A, const float *__restrict__ B,
                                                  float *__restrict__ C, int64_t M, int64_t K, int64_t N)
{
    __shared__ float As[3][TK][TM + 4];
    __shared__ float Bs[3][TK][TN + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t m0 = (int64_t)blockIdx.y * TM, n0 = (int64_t)blockIdx.x * TN;
    Acc acc[3][4][4];
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++)
                acc[c][i][j] = 0;
    for (int64_t k0 = 0; k0 < K; k0 += TK) {
        /* A tile: TM rows x TK k x 3 channels = 3072 floats; 12 per thread */
        for (int e = threadIdx.x; e < TM * TK * 3; e += 256) {
            int r = e / (TK * 3), rem = e - r * (TK * 3);
            int kk = rem / 3, c = rem - kk * 3;
            int64_t gm = m0 + r, gk = k0 + kk;
            As[c][kk][r] = (gm < M && gk < K) ? A[3 * (gm * K + gk) + c] : 0.f;
        }
        /* B tile: TK rows x TN columns x 3 channels */
        for (int e = threadIdx.x; e < TK * TN * 3; e += 256) {
            int kk = e / (TN * 3), rem = e - kk * (TN * 3);
            int col = rem / 3, c = rem - col * 3;
            int64_t gk = k0 + kk, gn = n0 + col;
            Bs[c][kk][col] = (gk < K && gn < N) ? B[3 * (gk * N + gn) + c] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < TK; kk++) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                float a[4], b[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    a[i] = As[c][kk][ty + 16 * i];
                    b[i] = Bs[c][kk][tx + 16 * i];
                }
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        acc[c][i][j] += (Acc)a[i] * (Acc)b[j];
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int64_t gm = m0 + ty + 16 * i;
        if (gm >= M)
            continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int64_t gn = n0 + tx + 16 * j;
            if (gn >= N)
                continue;
            float *o = C + 3 * (gm * N + gn);
            o[0] = (float)acc[0][i][j];
            o[1] = (float)acc[1][i][j];
            o[2] = (float)acc[2][i][j];
        }
    }
}

int gb_dct_device(const float *A, const float *B, int64_t M, int64_t K, int64_t N, int mode, float *C,
                  cudaStream_t st, std::string &err)
{
    if (M <= 0 || K <= 0 || N <= 0) {
        err = "bad matrix dimensions";
        return GB_EINVAL;
    }
    if (mode == GB_DCT_BF16X3 || mode == GB_DCT_FP16X3 || mode == GB_DCT_FP16)
        return gb_dct_tc(A, B, M, K, N, mode, C, st, err);
    dim3 grid((unsigned)((N + TN - 1) / TN), (unsigned)((M + TM - 1) / TM));
    if (grid.y > 65535) {
        err = "too many rows for one launch";
        return GB_EINVAL;
    }
    if (mode == GB_DCT_FP32)
        k_dct_simt<float><<<grid, 256, 0, st>>>(A, B, C, M, K, N);
    else if (mode == GB_DCT_FP64)
        k_dct_simt<double><<<grid, 256, 0, st>>>(A, B, C, M, K, N);
    else {
        err = "unknown dctimestep mode";
        return GB_EINVAL;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = cudaGetErrorString(e);
        return GB_ECUDA;
    }
    return 0;
}
