/*
 * dct_tc.cu -- dctimestep's product on the 5th-generation tensor cores,
 * BF16x3 split precision with FP32 accumulation.
 */
#include "dct.h"
#include "../../include/gbrad.h"

int gb_dct_bf16x3(const float *A, const float *B, int64_t M, int64_t K, int64_t N, float *C, cudaStream_t st,
                  std::string &err)
{
    (void)A; (void)B; (void)M; (void)K; (void)N; (void)C; (void)st;
    err = "the BF16x3 tensor-core product is not built yet";
    return GB_EUNSUPPORTED;
}
