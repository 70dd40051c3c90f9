/* Kernels of the design-screening surrogate network (ffip_gb300/surrogate.py):
 * no counterpart in the reference, which has no learned part.  All pointers
 * are DEVICE pointers of the calling process's current CUDA device; `stream`
 * is a cudaStream_t (NULL = the legacy default stream).  Return 0 or a
 * negative code (ffip_gb300.h) with the message in ffip_last_error(). */
#ifndef FFIP_GB300_SURROGATE_H
#define FFIP_GB300_SURROGATE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* C[M,N] = A[M,K] B[K,N] (+ bias[M]) in fp32, or C += that when accumulate
 * is non-zero.  A and B are bf16 with element (r, c) at p[r * rs + c * cs]
 * (any strides: transposes are stride swaps); C is fp32, same convention;
 * bias is fp32 or NULL.  Tensor cores (bf16 in, fp32 accumulate). */
int ffip_sg_gemm(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs,
                 float *C, int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream);

/* im2col of a bf16 tensor x[N][C][D][H][W] (shape5) for a convolution with
 * kernel3 (kd, kh, kw), stride3 and zero padding pad3: cols is bf16
 * [C*kd*kh*kw][N*Do*Ho*Wo], row (c, kd, kh, kw), column (n, od, oh, ow). */
int ffip_sg_im2col(const void *x, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, void *cols,
                   void *stream);

/* The transpose of ffip_sg_im2col on fp32 data: dx[N][C][D][H][W] is
 * overwritten with the sums of the dcols entries that read each element. */
int ffip_sg_col2im(const float *dcols, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, float *dx,
                   void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FFIP_GB300_SURROGATE_H */
