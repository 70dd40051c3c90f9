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
 * bias is fp32 or NULL.  Tensor cores (bf16 in, fp32 accumulate): operands
 * with K contiguous in both (acs == 1, brs == 1), row strides multiples of 8
 * elements and 16-byte aligned bases run on tcgen05 (TMA-fed, accumulator in
 * tensor memory), any other layout on mma.sync. */
int ffip_sg_gemm(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs,
                 float *C, int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream);

/* The same with the kernel chosen: path 0 as ffip_sg_gemm, 1 the tcgen05
 * kernel (an error for operands it does not take), 2 the mma.sync kernel. */
int ffip_sg_gemm_path(int M, int N, int K, const void *A, int64_t ars, int64_t acs, const void *B, int64_t brs, int64_t bcs,
                      float *C, int64_t crs, int64_t ccs, const float *bias, int accumulate, void *stream, int path);

/* Synchronises the current device and reports whether a tcgen05 GEMM since
 * the last check gave up on a bounded wait (FFIP_ERR_CUDA with the message;
 * the word is cleared). */
int ffip_sg_check(void);

/* im2col of a bf16 tensor x[N][C][D][H][W] (shape5) for a convolution with
 * kernel3 (kd, kh, kw), stride3 and zero padding pad3: cols is bf16
 * [C*kd*kh*kw][N*Do*Ho*Wo], row (c, kd, kh, kw), column (n, od, oh, ow). */
int ffip_sg_im2col(const void *x, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, void *cols,
                   void *stream);

/* The same columns transposed: colsT is bf16 [N*Do*Ho*Wo][C*kd*kh*kw] (the
 * forward GEMM's reduction index contiguous, as the tcgen05 kernel takes it). */
int ffip_sg_im2col_t(const void *x, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, void *colsT,
                     void *stream);

/* The transpose of ffip_sg_im2col on fp32 data: dx[N][C][D][H][W] is
 * overwritten with the sums of the dcols entries that read each element. */
int ffip_sg_col2im(const float *dcols, const int *shape5, const int *kernel3, const int *stride3, const int *pad3, float *dx,
                   void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FFIP_GB300_SURROGATE_H */
