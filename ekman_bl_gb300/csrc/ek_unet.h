// The U-Net of the learned Poisson initial guess (ek_unet.cu): host-side
// object owning the parameters, the Adam state and the activation and
// gradient buffers.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace ek {

class UNet {
 public:
  static constexpr int kLevels = 4;
  static constexpr int kLayers = 15;
  // cin input channels, C channels at every level, images of h x w pixels
  // (multiples of 8), at most max_n images per call.
  UNet(int cin, int C, int max_n, int h, int w);
  ~UNet();
  UNet(const UNet &) = delete;
  UNet &operator=(const UNet &) = delete;

  long nparams() const { return nparam_; }
  // Parameter layout, layer after layer: W[cout][9][cin] then b[cout].
  void set_params(const float *host);  // also resets the Adam state
  void get_params(float *host) const;
  void layer_shape(int l, int *cin, int *cout) const;

  // x: device FP32 [n][h][w][cin]; y: device FP32 [n][h][w]
  void forward(const float *x, int n, float *y, cudaStream_t s);
  // Forward, mean-square error against t over the top-left hv x wv pixels
  // of each image, backward; the parameter gradient lands in grads().
  double forward_backward(const float *x, const float *t, int n, int hv, int wv, float *y, cudaStream_t s);
  // forward_backward, then one Adam step (lr, beta1 0.9, beta2 0.999, eps 1e-8)
  double train_step(const float *x, const float *t, int n, int hv, int wv, double lr, cudaStream_t s);
  const float *grads() const { return grad_; }
  long launches() const { return launches_; }
  double forward_flops(int n) const;  // 2 x multiply-adds of the convolutions
  // the forward convolutions whose channel counts allow it on the tcgen05
  // kernel (default), else all on the mma.sync one
  void set_tcgen05(bool on) { tc_ = on; }
  bool tcgen05() const { return tc_; }
  // 1 when a tcgen05 convolution's bounded wait ran out (sticky); reads the
  // device flag (synchronises the stream)
  int tc_error(cudaStream_t s);

  int cin, C, max_n, h, w;

 private:
  struct Layer {
    int cin, cout, c1, c2;
    long woff, boff;
    int relu;
  };
  Layer L_[kLayers];
  long nparam_ = 0;
  float *param_ = nullptr, *grad_ = nullptr, *m_ = nullptr, *v_ = nullptr;
  long step_ = 0;
  long launches_ = 0;
  bool tc_ = true;
  int *tc_err_ = nullptr;
  // activations (BF16, bordered): xin, t[l], s[l], p[l], u[l], v[l], d[l]
  unsigned short *xin_ = nullptr;
  unsigned short *t_[kLevels] = {}, *s_[kLevels] = {}, *p_[kLevels] = {};
  unsigned short *u_[kLevels] = {}, *vv_[kLevels] = {}, *d_[kLevels] = {};
  float *y_ = nullptr;
  // gradients (FP32, bordered), allocated on the first backward pass
  int gn_ = 0;
  float *gy_ = nullptr;
  float *gt_[kLevels] = {}, *gs_[kLevels] = {}, *gp_[kLevels] = {};
  float *gu_[kLevels] = {}, *gv_[kLevels] = {}, *gd_[kLevels] = {};
  double *loss_ = nullptr;
  std::vector<void *> bufs_, gbufs_;

  void *alloc(size_t bytes, std::vector<void *> &list);
  void alloc_grads(int n);
  void run_forward(const float *x, int n, float *y, cudaStream_t s);
};

}  // namespace ek
