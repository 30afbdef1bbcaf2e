// scf_unet.cuh -- the U-Net of include/scf_unet.h as a C++ object, used by the
// C-ABI (training, tests) and by the projection solver (inference inside the
// flexible PCG).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

namespace scf {

// One 3x3 convolution (zero padding, bias) of NHWC BF16 tensors.
struct ConvArgs {
  const __nv_bfloat16* in;    // [n][Hi][Wi][CIN]; Hi = H/2, Wi = W/2 when upsampling
  const __nv_bfloat16* mask;  // backward of a ReLU layer: [n][H][W][CIN], input used where > 0
  const __nv_bfloat16* wt;    // [COUT][9][CIN]
  const float* bias;          // [COUT] or null
  const __nv_bfloat16* add;   // skip tensor [n][H][W][COUT] added to the output, or null
  __nv_bfloat16* out;         // [n][H][W][COUT]
  int n, H, W;
};

// The convolution on the tcgen05 tensor cores (scf_unet_tc.cu).  Forward
// (bwd = false): ups -> nearest-upsampled input plus skip add, else ReLU
// output.  Input gradient (bwd = true, cin/cout the layer's cout/cin): mask ->
// input masked by the ReLU output.  *err (device int) is set when a bounded
// wait runs out.  Returns 0, or -1 for a channel pair or variant that the
// network does not have or a failed launch.
// map: device copy of the input's tensor map from conv_tma_map, or null.
// With a map the forward layers (ReLU layers of 32 or 64 channels on a side,
// upsampling layers) stage their input rows by TMA.
int conv_tc(int cin, int cout, const ConvArgs& a, bool ups, bool bwd, bool mask, int sms,
            int* err, const CUtensorMap* map, cudaStream_t s);
// Tensor map of an NHWC BF16 tensor [n][H][W][cin] for the TMA-staged
// convolution (host; 0 on success).  The input of an upsampling layer is
// mapped with its own (half-resolution) dimensions.
int conv_tma_map(CUtensorMap* m, const void* in, int n, int H, int W, int cin);

struct UNetLayer {
  int cin, cout;  // channels in / out
  int level;      // resolution level of the output (0 = full)
  bool ups;       // input read at half resolution (nearest upsampling)
  bool relu;      // ReLU on the output
  int skip;       // layer whose output is added to this one's (-1: none)
  size_t woff, boff;  // offsets of W ([cout][9][cin]) and bias in the parameters
};

class UNet {
 public:
  // batch n of h x w images (multiples of 8); train: also the backward buffers
  int create(int n, int h, int w, bool train, int device);
  void destroy();
  ~UNet() { destroy(); }

  static int num_params();
  static const std::vector<UNetLayer>& layers();

  // parameters: host FP32 array in the order of include/scf_unet.h
  int set_params_host(const float* p);
  int get_params_host(float* p);

  // input features of image i from FP64 device arrays with cell (x, y) at
  // y * ld + x; sigma_out (device float) gets the residual scale
  void features(int i, int nx, int ny, int ld, const double* r, const double* cE,
                const double* cN, const double* dg, float* sigma_out, cudaStream_t s);
  void forward(cudaStream_t s);  // leaves z (n*h*w FP32) in z_
  // FP32 correction on a padded level layout: x[g] = sigma * z on cells with dg > 0
  void correction(int nx, int ny, int pitch, const double* dg, const float* sigma, float* x,
                  cudaStream_t s);
  // training target of image i: t = e / sigma, mask = dg > 0 (Fortran (nx,ny) arrays)
  void target(int i, int nx, int ny, const double* e, const double* dg, const float* sigma,
              float* t, unsigned char* mask, cudaStream_t s);
  void loss(const float* t, const unsigned char* mask, float* loss_dev, cudaStream_t s);
  void backward(cudaStream_t s);
  void adam(float lr, float b1, float b2, float eps, int step, cudaStream_t s);
  void refresh_weights(cudaStream_t s);  // BF16 copies after a parameter change

  int n_ = 0, h_ = 0, w_ = 0;
  bool train_ = false;
  // convolution engine: 1 = tcgen05 (TMEM accumulators) with the forward
  // ReLU layers' rows staged by TMA, 2 = tcgen05 with every row staged by
  // the threads, 0 = mma.sync (kept as the comparison for tests and
  // measurements); weight gradients use mma.sync either way
  int engine_ = 1;
  CUtensorMap* maps_ = nullptr;  // device: tensor map of each layer's input (forward)
  std::vector<char> has_map_;    // the layer's map was accepted
  int* tc_err_ = nullptr;  // device flag: a tcgen05 convolution's bounded wait ran out
  int sms_ = 152;
  float *params_ = nullptr, *grads_ = nullptr, *m_ = nullptr, *v_ = nullptr;
  __nv_bfloat16 *wb_ = nullptr, *wt_ = nullptr;  // BF16 weights and flipped transposes
  float *z_ = nullptr, *dz_ = nullptr, *red_ = nullptr;
  __nv_bfloat16* in_ = nullptr;            // input features [n][h][w][16]
  std::vector<__nv_bfloat16*> act_;        // layer outputs
  std::vector<__nv_bfloat16*> pool_;       // pooled inputs of e1a, e2a, e3a
  std::vector<__nv_bfloat16*> g_;          // scratch gradient buffers
  std::vector<void*> allocs_;

 private:
  int alloc(void** p, size_t bytes);
};

}  // namespace scf
