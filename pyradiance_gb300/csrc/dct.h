/* dct.h -- dctimestep matrix product kernels (dct.cu, dct_tc.cu) */
#ifndef GB_DCT_H
#define GB_DCT_H

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

/* R[m,n,c] = sum_k A[m,k,c] * B[k,n,c], interleaved RGB float32 operands on
 * the device.  Returns 0 or a negative GB_E* code with err set. */
int gb_dct_device(const float *A, const float *B, int64_t M, int64_t K, int64_t N, int mode, float *C,
                  cudaStream_t st, std::string &err);

/* tensor-core forms (dct_tc.cu): GB_DCT_BF16X3, GB_DCT_FP16X3, GB_DCT_FP16 */
int gb_dct_tc(const float *A, const float *B, int64_t M, int64_t K, int64_t N, int mode, float *C,
              cudaStream_t st, std::string &err);

#endif
