// The learned mode's network: sizes, device parameter view, trainer.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace ho {

constexpr int kMlpIn = 48;      // 8 corners + 6 face-centre offsets (42) + entry point (3) + direction (3)
constexpr int kMlpInPad = 64;   // rows of X are padded with zeros to 64 BF16
constexpr int kMlpHidden = 128;
constexpr int kMlpOut = 8;      // xi at the segment entry (3) + d xi / d t there (3) + 2 unused
constexpr int kMlpTargets = 6;  // outputs that carry a training target
constexpr int kMlpParams = kMlpIn * kMlpHidden + kMlpHidden + 2 * (kMlpHidden * kMlpHidden + kMlpHidden) +
                           kMlpHidden * kMlpOut + kMlpOut;

// BF16 transposed weights (Wt[out][in]) and FP32 biases for inference.
struct MlpDev {
  const void* w1t;  // [128][64]
  const void* w2t;  // [128][128]
  const void* w3t;  // [128][128]
  const void* w4t;  // [16][128] (rows 8..15 zero)
  const float* b1;
  const float* b2;
  const float* b3;
  const float* b4;
};

struct Mlp {
  // per layer l: W[l] is [in][out] row-major FP32 master; Wb BF16 copy
  float* W[4] = {nullptr, nullptr, nullptr, nullptr};
  void* Wb[4] = {nullptr, nullptr, nullptr, nullptr};
  float* gW[4] = {nullptr, nullptr, nullptr, nullptr};
  float* mW[4] = {nullptr, nullptr, nullptr, nullptr};
  float* vW[4] = {nullptr, nullptr, nullptr, nullptr};
  float* b[4] = {nullptr, nullptr, nullptr, nullptr};
  float* gb[4] = {nullptr, nullptr, nullptr, nullptr};
  float* mb[4] = {nullptr, nullptr, nullptr, nullptr};
  float* vb[4] = {nullptr, nullptr, nullptr, nullptr};
  void* wt[4] = {nullptr, nullptr, nullptr, nullptr};
  void* ws = nullptr;
  int ws_rows = 0;
  int step = 0;
  bool ready = false;
  bool trained = false;

  int alloc();
  void release();
  int set_params(const float* const* Wh, const float* const* bh, cudaStream_t s);
  int get_params(float* const* Wh, float* const* bh, cudaStream_t s);
  int refresh_copies(cudaStream_t s);
  MlpDev dev() const;
  int ensure_ws(int rows);
  int forward_backward(int B, const void* Xb, const float* Tb, const uint8_t* Vb, int n_valid, float* loss_dev,
                       cudaStream_t s);
  int adam_step(float lr, cudaStream_t s);
  int train(const void* X, const float* T, const uint8_t* V, int64_t n, int steps, int batch, float lr, uint64_t seed,
            std::vector<float>& losses, cudaStream_t s);
  // pointers into the workspace after forward_backward (for gradient checks)
};

size_t mlp_infer_smem();
// Y[rows x 8] = MLP(X[rows x 64]); rows = m_dev ? (*m_dev) * rows_per_item : M.
int mlp_infer(const MlpDev& P, const void* X, int64_t M, const unsigned* m_dev, int rows_per_item, float* Y,
              cudaStream_t s, int grid);

}  // namespace ho
