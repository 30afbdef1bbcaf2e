/*
 * scf_unet.h -- the learned preconditioner of the projection solver: a small
 * U-Net that maps the PCG residual and the face couplings of the pressure
 * operator to a correction.  No reference counterpart: the reference solves
 * with HYPRE PCG + BoomerAMG (src/ProjectionP_Mod.f90:101-135); this network
 * is an optional preconditioner of the flexible PCG that replaces it, with
 * the multigrid V-cycle as the fallback (scf_proj_set_network in scf_proj.h).
 *
 * Network (about 0.26 M parameters), NHWC BF16 activations, FP32
 * accumulation on the tensor cores: the forward convolutions and the input
 * gradients on tcgen05.mma with the accumulators in tensor memory, the
 * weight gradients on mma.sync m16n8k16:
 *   level 0 (H x W, 16 ch):  e0a = relu(conv(in)),  e0 = relu(conv(e0a))
 *   level 1 (H/2, 32 ch):    e1a = relu(conv(pool(e0))), e1 = relu(conv(e1a))
 *   level 2 (H/4, 64 ch):    e2a = relu(conv(pool(e1))), e2 = relu(conv(e2a))
 *   level 3 (H/8, 64 ch):    e3a = relu(conv(pool(e2))), e3 = relu(conv(e3a))
 *   decoder, additive skips: u2 = conv(up(e3)) + e2,  d2 = relu(conv(u2))
 *                            u1 = conv(up(d2)) + e1,  d1 = relu(conv(u1))
 *                            u0 = conv(up(d1)) + e0,  d0 = relu(conv(u0))
 *   head: z = w . d0 + b (1x1 convolution, 16 -> 1)
 * conv = 3x3, zero padding, with bias; pool = 2x2 mean; up = nearest.
 * Input features per cell (channels 5..15 are zero):
 *   0: r/dg / sigma  (sigma = RMS of r/dg over cells with an unknown)
 *   1: cE/dg, 2: cE(west face)/dg, 3: cN/dg, 4: cN(south face)/dg
 * and the correction is z * sigma on cells with an unknown.
 *
 * Parameters (FP32 master copy, in this order, per layer W then bias):
 *   layers e0a e0 e1a e1 e2a e2 e3a e3 u2 d2 u1 d1 u0 d0, W as [Cout][3][3][Cin],
 *   then the head weights [16] and bias [1].
 */
#ifndef SCF_UNET_H
#define SCF_UNET_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct scf_unet scf_unet;

/* Number of FP32 parameters. */
int scf_unet_num_params(void);

/* A network instance for a batch of n images of h x w cells (h, w multiples
 * of 8), with all activation and gradient buffers, on the given device. */
int scf_unet_create(scf_unet **u, int n, int h, int w, int device);
int scf_unet_destroy(scf_unet *u);
int scf_unet_set_stream(scf_unet *u, void *stream);

/* Parameters: host arrays of scf_unet_num_params() floats. */
int scf_unet_set_params(scf_unet *u, const float *params);
int scf_unet_get_params(scf_unet *u, float *params);

/* Input features of image i from an operator and a residual given as
 * device arrays in Fortran (nx, ny) order with nx <= w, ny <= h (the rest of
 * the image is zero): r, cE, cN, dg (dg <= 0: no unknown).  sigma_out: device
 * float receiving sigma of image i. */
int scf_unet_features(scf_unet *u, int i, int nx, int ny, const double *r, const double *cE,
                      const double *cN, const double *dg, float *sigma_out);

/* Training target of image i: t[i] = e / sigma (sigma from
 * scf_unet_features of the same image) and mask[i] = dg > 0, with e, dg
 * device arrays in Fortran (nx, ny) order; t (n*h*w floats) and mask
 * (n*h*w bytes) are device arrays for the whole batch. */
int scf_unet_target(scf_unet *u, int i, int nx, int ny, const double *e, const double *dg,
                    const float *sigma, float *t, unsigned char *mask);

/* Raw input (host, n*h*w*5 floats, NHWC with 5 channels), for tests. */
int scf_unet_set_input(scf_unet *u, const float *x);

/* Convolution engine of the forward pass and the input gradients:
 * 1 = tcgen05 with the forward layers' input rows staged by TMA
 * (default), 2 = tcgen05 with every input row staged by the CTA's threads,
 * 0 = the mma.sync kernels (comparison only). */
int scf_unet_set_engine(scf_unet *u, int engine);

/* Forward pass; z: n*h*w floats (device pointer when device != 0).
 * Returns -3 if a tcgen05 convolution's bounded wait ran out. */
int scf_unet_forward(scf_unet *u, float *z, int device);

/* One 3x3 convolution of the network on device arrays, for tests and
 * measurements: NHWC BF16 in [n][H][W][cin] (half resolution with ups),
 * wt BF16 [cout][9][cin], bias FP32 [cout], out BF16 [n][H][W][cout].
 * Variants as the network uses them: forward with ReLU (ups = bwd = mask =
 * 0), forward with nearest upsampling of `in` and the skip tensor `add`
 * [n][H][W][cout] added (ups = 1, no ReLU), input gradient (bwd = 1, bias
 * and add null) with `in` masked by maskp > 0 (mask = 1) or not.  Engine as
 * scf_unet_set_engine; stream: a cudaStream_t or null.  Returns 0, -1 for
 * arguments outside these variants, -2 for a CUDA error, -3 for a bounded
 * wait that ran out. */
int scf_unet_conv(int engine, int cin, int cout, int ups, int bwd, int mask, const void *in,
                  const void *maskp, const void *wt, const float *bias, const void *add,
                  void *out, int n, int H, int W, void *stream);

/* Loss of the last forward pass against the target t (device, n*h*w
 * floats) on the cells where mask (device, n*h*w bytes) is nonzero:
 *   L = sum_i sum_p (z - t)^2 / sum_p t^2 (per image normalised)
 * leaves dL/dz in the network; loss_out: host float. */
int scf_unet_loss(scf_unet *u, const float *t, const unsigned char *mask, float *loss_out);

/* Set dL/dz directly (host, n*h*w floats), for tests. */
int scf_unet_set_dz(scf_unet *u, const float *dz);

/* Backward pass from dL/dz: parameter gradients (FP32). */
int scf_unet_backward(scf_unet *u);
int scf_unet_get_grads(scf_unet *u, float *grads);

/* One Adam step on the parameters with the current gradients (step >= 1). */
int scf_unet_adam(scf_unet *u, float lr, float beta1, float beta2, float eps, int step);

#ifdef __cplusplus
}
#endif

#endif /* SCF_UNET_H */
