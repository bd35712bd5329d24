/*
 * imexlb_nn.h -- tensor-core kernels of the warm-start neural operator (no
 * counterpart in the reference). A small convolutional encoder-decoder maps
 * an obstacle mask and the Reynolds number to an initial (p, u) field for the
 * lattice Boltzmann solver; these entry points are its forward and backward
 * passes and its optimiser, on caller-owned device memory.
 *
 * The convolutions run on the tcgen05 tensor cores (bf16 operands staged in
 * shared memory, FP32 accumulation in tensor memory).
 *
 * Layout: activations NHWC bfloat16 (channels innermost); weights
 * w[co][tap*Cin + ci] bfloat16 with tap = ky*3 + kx; FP32 accumulation.
 * Cin and Cout must be multiples of 16 (pad with zero channels).
 * All calls enqueue on `stream` (a cudaStream_t, NULL for the default
 * stream) and return 0, -1 (bad argument) or -2 (launch error).
 */
#ifndef IMEXLB_NN_H
#define IMEXLB_NN_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct imexlb_conv_desc {
  int n;            /* images */
  int hin, win;     /* input size */
  int cin;          /* input channels (multiple of 16) */
  int hout, wout;   /* output size: ((up?2:1)*hin - 1)/stride + 1 */
  int cout;         /* output channels of the GEMM (multiple of 16, <= 64) */
  int cout_store;   /* channels written per output pixel (0: cout) */
  int stride;       /* 1 or 2 */
  int upsample;     /* 1: the 3x3 stencil runs on the input upsampled x2 (nearest) */
} imexlb_conv_desc;

/* y = act(conv3x3(x) + bias), act = ReLU when relu != 0; y bf16 (y_bf16) or
 * f32 (y_f32), cout_store channels per pixel. */
int imexlb_nn_conv_fwd(const imexlb_conv_desc* d, const void* x, const void* w, const float* bias,
                       int relu, void* y_bf16, float* y_f32, void* stream);

/* dz = bf16(dy * relu'(y)) for n = pixels*c values (relu = 0: dz = dy), and
 * dbias[c] += column sums of dz (dbias may be NULL). */
int imexlb_nn_act_grad(const float* dy, const void* y, long long n, int c, int relu, void* dz,
                       float* dbias, void* stream);

/* Gradient with respect to the input: dgrid (f32, the stencil grid, i.e. the
 * upsampled input when upsample) and, when upsample, dx (f32, summed over
 * each pixel's 2x2 children). wt_scratch: 9*cin*cout bf16 of caller memory. */
int imexlb_nn_conv_bwd_data(const imexlb_conv_desc* d, const void* dz, const void* w, void* wt_scratch,
                            float* dgrid, float* dx, void* stream);

/* dw[co][tap*Cin + ci] += sum over output pixels of dz * im2col(x) (f32). */
int imexlb_nn_conv_bwd_weight(const imexlb_conv_desc* d, const void* x, const void* dz, float* dw,
                              void* stream);

/* Mean squared error between y (npix x c, f32) and target (npix x used) over
 * the first `used` channels, optionally weighted per pixel; *loss += mean,
 * dy (npix x c) = d(loss)/dy with zeros in the padding channels. */
int imexlb_nn_mse(const float* y, const float* target, const float* weight, long long npix, int c,
                  int used, float* dy, float* loss, void* stream);

/* Adam (with L2 weight decay added to the gradient) on f32 master weights p;
 * p_bf16 (may be NULL) receives the rounded copy the convolutions read.
 * t = step number starting at 1. */
int imexlb_nn_adam(float* p, const float* g, float* m, float* v, void* p_bf16, long long n, float lr,
                   float beta1, float beta2, float eps, int t, float weight_decay, void* stream);

/* Status of the convolution kernels since the last call: 0, or 1 when a
 * kernel gave up waiting for its tensor-core work (a bounded wait; the
 * results of that launch are then incomplete). Reading clears it. */
int imexlb_nn_status(int* status);

#ifdef __cplusplus
}
#endif
#endif /* IMEXLB_NN_H */
