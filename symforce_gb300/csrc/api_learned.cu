// C ABI of the camera-block preconditioner network: training (Adam over shuffled mini-batches),
// one forward + backward pass for gradient checks, and inference.  All arithmetic runs in the
// hand-written kernels of kernels_mlp.cu / kernels_pcg.cu on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "device_plan.h"
#include "kernels.h"

namespace sfg {
extern thread_local std::string g_last_error;

namespace {

struct NetPtrs {
  float *W1, *b1, *W2, *b2, *W3, *b3;
};

NetPtrs Split(float* w) {
  NetPtrs p;
  p.W1 = w;
  p.b1 = p.W1 + kPrecondFeatures * kPrecondHidden;
  p.W2 = p.b1 + kPrecondHidden;
  p.b2 = p.W2 + kPrecondHidden * kPrecondHidden;
  p.W3 = p.b2 + kPrecondHidden;
  p.b3 = p.W3 + kPrecondHidden * kPrecondTri;
  return p;
}

// Activations and gradients for up to `cap` samples.
struct Workspace {
  int cap = 0;
  float *H1, *H2, *Z, *dZ, *dH2, *dH1, *loss;
  int* err;  // set by a tensor-core GEMM whose capped wait gave up
  void Init(DeviceArena& A, int n) {
    cap = n;
    err = A.Zeros<int>(1);
    H1 = static_cast<float*>(A.Alloc(size_t(n) * kPrecondHidden * 4));
    H2 = static_cast<float*>(A.Alloc(size_t(n) * kPrecondHidden * 4));
    Z = static_cast<float*>(A.Alloc(size_t(n) * kPrecondTri * 4));
    dZ = static_cast<float*>(A.Alloc(size_t(n) * kPrecondTri * 4));
    dH2 = static_cast<float*>(A.Alloc(size_t(n) * kPrecondHidden * 4));
    dH1 = static_cast<float*>(A.Alloc(size_t(n) * kPrecondHidden * 4));
    loss = static_cast<float*>(A.Alloc(size_t(n) * 4));
  }
};

// Mean loss of n sample rows (row stride kSampleFloats) into *loss_sum and its gradient into g.
void ForwardBackward(const Workspace& ws, float* weights, float* grad, const float* rows, int n,
                     float kaporin, double* loss_sum, cudaStream_t s) {
  const NetPtrs w = Split(weights);
  const NetPtrs g = Split(grad);
  const int F = kPrecondFeatures, H = kPrecondHidden, O = kPrecondTri;
  const int64_t ld = kSampleFloats;
  // every product on the tensor cores (tcgen05, TF32 with the three-pass FP32 split)
  SFG_CUDA(LaunchGemmTc(n, H, F, rows, ld, 1, w.W1, H, 1, ws.H1, H, kEpiBiasRelu, w.b1, nullptr, 0, ws.err, s));
  SFG_CUDA(LaunchGemmTc(n, H, H, ws.H1, H, 1, w.W2, H, 1, ws.H2, H, kEpiBiasRelu, w.b2, nullptr, 0, ws.err, s));
  SFG_CUDA(LaunchGemmTc(n, O, H, ws.H2, H, 1, w.W3, O, 1, ws.Z, O, kEpiBias, w.b3, nullptr, 0, ws.err, s));
  LaunchHead(n, ws.Z, rows, ld, 1.f / float(n), kaporin, ws.dZ, ws.loss, loss_sum, s);
  SFG_CUDA(LaunchGemmTc(H, O, n, ws.H2, 1, H, ws.dZ, O, 1, g.W3, O, kEpiNone, nullptr, nullptr, 0, ws.err, s));
  LaunchColSum(n, O, ws.dZ, O, g.b3, s);
  SFG_CUDA(LaunchGemmTc(n, H, O, ws.dZ, O, 1, w.W3, 1, O, ws.dH2, H, kEpiMask, nullptr, ws.H2, H, ws.err, s));
  SFG_CUDA(LaunchGemmTc(H, H, n, ws.H1, 1, H, ws.dH2, H, 1, g.W2, H, kEpiNone, nullptr, nullptr, 0, ws.err, s));
  LaunchColSum(n, H, ws.dH2, H, g.b2, s);
  SFG_CUDA(LaunchGemmTc(n, H, H, ws.dH2, H, 1, w.W2, 1, H, ws.dH1, H, kEpiMask, nullptr, ws.H1, H, ws.err, s));
  SFG_CUDA(LaunchGemmTc(F, H, n, rows, 1, ld, ws.dH1, H, 1, g.W1, H, kEpiNone, nullptr, nullptr, 0, ws.err, s));
  LaunchColSum(n, H, ws.dH1, H, g.b1, s);
}

template <typename F>
int32_t GuardL(F&& fn) {
  try {
    fn();
    return SFG_OK;
  } catch (const Error& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host out of memory";
    return SFG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return SFG_ERR_INVALID_ARGUMENT;
  }
}

void CheckErr(const int* err) {
  int e = 0;
  SFG_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) throw Error(SFG_ERR_DEVICE_STATUS, "tensor-core GEMM: a wait hit its cap");
}

void UseDevice(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    throw Error(SFG_ERR_NO_DEVICE, "no CUDA device is visible; this library has no CPU fallback");
  if (device < 0 || device >= n) throw Error(SFG_ERR_INVALID_ARGUMENT, "bad device ordinal");
  SFG_CUDA(cudaSetDevice(device));
}

struct Stream {
  cudaStream_t s = nullptr;
  Stream() { SFG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~Stream() {
    if (s) cudaStreamDestroy(s);
  }
};

}  // namespace
}  // namespace sfg

using sfg::Error;

extern "C" {

int32_t sfg_precond_train(const float* samples, int64_t n, const sfg_train_params_t* params,
                          float* weights, float* loss_curve) {
  return sfg::GuardL([&] {
    if (!samples || !params || !weights || n <= 0)
      throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument or no samples");
    if (n > (int64_t(1) << 31) - 1) throw Error(SFG_ERR_INVALID_ARGUMENT, "too many samples");
    const sfg_train_params_t& p = *params;
    if (p.steps <= 0 || p.batch <= 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "steps and batch must be positive");
    if (!(p.kaporin >= 0.f)) throw Error(SFG_ERR_INVALID_ARGUMENT, "kaporin must be >= 0");
    sfg::UseDevice(p.device);
    const int B = int(std::min<int64_t>(p.batch, n));
    sfg::DeviceArena A;
    sfg::Stream st;
    cudaStream_t s = st.s;
    float* d_samples = static_cast<float*>(A.Alloc(size_t(n) * sfg::kSampleFloats * 4));
    SFG_CUDA(cudaMemcpy(d_samples, samples, size_t(n) * sfg::kSampleFloats * 4, cudaMemcpyHostToDevice));
    const size_t P = sfg::kPrecondParams;
    float* w = static_cast<float*>(A.Alloc(P * 4));
    SFG_CUDA(cudaMemcpy(w, weights, P * 4, cudaMemcpyHostToDevice));
    float* g = A.Zeros<float>(P);
    float* m = A.Zeros<float>(P);
    float* v = A.Zeros<float>(P);
    float* rows = static_cast<float*>(A.Alloc(size_t(B) * sfg::kSampleFloats * 4));
    int32_t* idx = static_cast<int32_t*>(A.Alloc(size_t(n) * 4));
    double* losses = A.Zeros<double>(size_t(p.steps));
    sfg::Workspace ws;
    ws.Init(A, B);
    std::vector<int32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::mt19937_64 rng(p.seed);
    int64_t pos = n;  // forces a shuffle before the first step
    const float beta1 = p.beta1 > 0 ? p.beta1 : 0.9f, beta2 = p.beta2 > 0 ? p.beta2 : 0.999f;
    const float eps = p.eps > 0 ? p.eps : 1e-8f;
    double b1t = 1.0, b2t = 1.0;
    for (int step = 0; step < p.steps; ++step) {
      if (pos + B > n) {
        for (int64_t i = n - 1; i > 0; --i) {
          const int64_t j = int64_t(rng() % uint64_t(i + 1));
          std::swap(perm[i], perm[j]);
        }
        SFG_CUDA(cudaMemcpyAsync(idx, perm.data(), size_t(n) * 4, cudaMemcpyHostToDevice, s));
        SFG_CUDA(cudaStreamSynchronize(s));
        pos = 0;
      }
      sfg::LaunchGather(B, d_samples, idx + pos, rows, s);
      pos += B;
      sfg::ForwardBackward(ws, w, g, rows, B, p.kaporin, losses + step, s);
      b1t *= beta1;
      b2t *= beta2;
      const double frac = p.steps > 1 ? double(step) / double(p.steps - 1) : 0.0;
      const float lr = float(p.lr * (0.1 + 0.9 * 0.5 * (1.0 + std::cos(M_PI * frac))));
      sfg::LaunchAdam(int64_t(P), w, g, m, v, lr, beta1, beta2, eps, float(1.0 - b1t), float(1.0 - b2t), s);
    }
    SFG_CUDA(cudaGetLastError());
    SFG_CUDA(cudaStreamSynchronize(s));
    sfg::CheckErr(ws.err);
    SFG_CUDA(cudaMemcpy(weights, w, P * 4, cudaMemcpyDeviceToHost));
    if (loss_curve) {
      std::vector<double> l(p.steps);
      SFG_CUDA(cudaMemcpy(l.data(), losses, size_t(p.steps) * 8, cudaMemcpyDeviceToHost));
      for (int i = 0; i < p.steps; ++i) loss_curve[i] = float(l[i]);
    }
  });
}

int32_t sfg_precond_loss_grad(const float* samples, int64_t n, const float* weights, float kaporin,
                              double* loss, float* grad, int32_t device) {
  return sfg::GuardL([&] {
    if (!samples || !weights || n <= 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument or no samples");
    if (n > (int64_t(1) << 24)) throw Error(SFG_ERR_INVALID_ARGUMENT, "too many samples for one pass");
    sfg::UseDevice(device);
    sfg::DeviceArena A;
    sfg::Stream st;
    cudaStream_t s = st.s;
    float* rows = static_cast<float*>(A.Alloc(size_t(n) * sfg::kSampleFloats * 4));
    SFG_CUDA(cudaMemcpy(rows, samples, size_t(n) * sfg::kSampleFloats * 4, cudaMemcpyHostToDevice));
    const size_t P = sfg::kPrecondParams;
    float* w = static_cast<float*>(A.Alloc(P * 4));
    SFG_CUDA(cudaMemcpy(w, weights, P * 4, cudaMemcpyHostToDevice));
    float* g = A.Zeros<float>(P);
    double* l = A.Zeros<double>(1);
    sfg::Workspace ws;
    ws.Init(A, int(n));
    sfg::ForwardBackward(ws, w, g, rows, int(n), kaporin, l, s);
    SFG_CUDA(cudaGetLastError());
    SFG_CUDA(cudaStreamSynchronize(s));
    sfg::CheckErr(ws.err);
    if (loss) SFG_CUDA(cudaMemcpy(loss, l, 8, cudaMemcpyDeviceToHost));
    if (grad) SFG_CUDA(cudaMemcpy(grad, g, P * 4, cudaMemcpyDeviceToHost));
  });
}

int32_t sfg_precond_infer(const float* features, int64_t n, const float* weights, float* out,
                          int32_t device) {
  return sfg::GuardL([&] {
    if (!features || !weights || !out || n <= 0) throw Error(SFG_ERR_INVALID_ARGUMENT, "null argument");
    sfg::UseDevice(device);
    sfg::DeviceArena A;
    sfg::Stream st;
    cudaStream_t s = st.s;
    float* x = static_cast<float*>(A.Alloc(size_t(n) * sfg::kPrecondFeatures * 4));
    SFG_CUDA(cudaMemcpy(x, features, size_t(n) * sfg::kPrecondFeatures * 4, cudaMemcpyHostToDevice));
    float* w = static_cast<float*>(A.Alloc(sfg::kPrecondParams * 4));
    SFG_CUDA(cudaMemcpy(w, weights, sfg::kPrecondParams * 4, cudaMemcpyHostToDevice));
    float* z = static_cast<float*>(A.Alloc(size_t(n) * sfg::kPrecondTri * 4));
    float* h1 = static_cast<float*>(A.Alloc(size_t(n) * sfg::kPrecondHidden * 4));
    float* h2 = static_cast<float*>(A.Alloc(size_t(n) * sfg::kPrecondHidden * 4));
    int* err = A.Zeros<int>(1);
    if (n > (int64_t(1) << 30)) throw Error(SFG_ERR_INVALID_ARGUMENT, "too many inputs for one pass");
    SFG_CUDA(sfg::LaunchMlpInferTc(x, sfg::kPrecondFeatures, n, w, h1, h2, z, err, s));
    SFG_CUDA(cudaStreamSynchronize(s));
    int e = 0;
    SFG_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) throw Error(SFG_ERR_DEVICE_STATUS, "tensor-core inference: a wait hit its cap");
    SFG_CUDA(cudaMemcpy(out, z, size_t(n) * sfg::kPrecondTri * 4, cudaMemcpyDeviceToHost));
  });
}

}  // extern "C"
