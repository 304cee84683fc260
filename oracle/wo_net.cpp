// TEST INFRASTRUCTURE ONLY: CPU restatement of one training step of the warm-start network, against
// which the tests compare the library's waves_net_gradients.  The network has no reference
// counterpart: 4 layers of 3x3x3 convolutions (3 -> 16 -> 16 -> 16 -> 1 channels), ReLU after the
// first three, zero padding at the crop edge; inputs, weights and the activations between layers
// are rounded to BF16 (round to nearest even) as in the inference kernels, accumulation is FP32.
//
// Layout: x[b][3][z][y][x], target and mask [b][z][y][x]; weights [co][27][ci] with tap
// t = (kz * 3 + ky) * 3 + kx at offset (kx - 1, ky - 1, kz - 1); biases [co].
// Loss: sum mask (y - target)^2 / max(sum mask, 1).  Backward: the exact gradient of that loss for
// the rounded forward (the roundings pass gradients through unchanged).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int kLayers = 4;
constexpr int kIn[kLayers] = {3, 16, 16, 16};
constexpr int kOut[kLayers] = {16, 16, 16, 1};

float bf16(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return v;  // inf / nan unchanged
  u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

struct Shape {
  int B, nz, ny, nx;
  size_t cells() const { return (size_t)nz * ny * nx; }
  long long at(int x, int y, int z) const { return ((long long)z * ny + y) * nx + x; }
};

// z[b][co][cell] = bias + sum_t sum_ci w[co][t][ci] a[b][ci][cell + off_t]
void forward_layer(const Shape& S, int ci_n, int co_n, const std::vector<float>& a, const std::vector<float>& w,
                   const float* bias, std::vector<float>& z) {
  const size_t C = S.cells();
  z.assign((size_t)S.B * co_n * C, 0.f);
#pragma omp parallel for collapse(2) schedule(static)
  for (int b = 0; b < S.B; b++)
    for (int co = 0; co < co_n; co++)
      for (int zz = 0; zz < S.nz; zz++)
        for (int yy = 0; yy < S.ny; yy++)
          for (int xx = 0; xx < S.nx; xx++) {
            float acc = bias[co];
            for (int t = 0; t < 27; t++) {
              const int qx = xx + t % 3 - 1, qy = yy + (t / 3) % 3 - 1, qz = zz + t / 9 - 1;
              if (qx < 0 || qy < 0 || qz < 0 || qx >= S.nx || qy >= S.ny || qz >= S.nz) continue;
              for (int ci = 0; ci < ci_n; ci++)
                acc += w[((size_t)co * 27 + t) * ci_n + ci] * a[((size_t)b * ci_n + ci) * C + S.at(qx, qy, qz)];
            }
            z[((size_t)b * co_n + co) * C + S.at(xx, yy, zz)] = acc;
          }
}

}  // namespace

extern "C" {

// One forward and backward pass: the loss, dL/dW and dL/db of every layer (FP32 weights in, the
// forward using their BF16 roundings), and the network output y[b][z][y][x].
double wo_net_gradients(int B, int nz, int ny, int nx, const float* x, const float* target, const float* mask,
                        const float* const* weights, const float* const* bias, float* const* gw, float* const* gb,
                        float* y_out) {
  const Shape S{B, nz, ny, nx};
  const size_t C = S.cells();
  std::vector<float> wb[kLayers];
  for (int l = 0; l < kLayers; l++) {
    wb[l].resize((size_t)kOut[l] * 27 * kIn[l]);
    for (size_t k = 0; k < wb[l].size(); k++) wb[l][k] = bf16(weights[l][k]);
  }
  std::vector<float> a[kLayers + 1], z[kLayers];
  a[0].resize((size_t)B * 3 * C);
  for (size_t k = 0; k < a[0].size(); k++) a[0][k] = bf16(x[k]);
  for (int l = 0; l < kLayers; l++) {
    forward_layer(S, kIn[l], kOut[l], a[l], wb[l], bias[l], z[l]);
    if (l + 1 < kLayers) {
      a[l + 1].resize(z[l].size());
      for (size_t k = 0; k < z[l].size(); k++) a[l + 1][k] = bf16(z[l][k] > 0.f ? z[l][k] : 0.f);
    }
  }
  double msum = 0.0, loss = 0.0;
  for (size_t k = 0; k < (size_t)B * C; k++) msum += mask[k];
  const double norm = msum > 1.0 ? msum : 1.0;
  std::vector<float> g((size_t)B * C);
  for (size_t k = 0; k < (size_t)B * C; k++) {
    const double d = (double)z[3][k] - (double)target[k];
    loss += mask[k] * d * d;
    g[k] = (float)(2.0 * mask[k] * d / norm);
    if (y_out) y_out[k] = z[3][k];
  }
  loss /= norm;
  // backward: g holds dL/dz of layer l
  for (int l = kLayers - 1; l >= 0; l--) {
    const int ci_n = kIn[l], co_n = kOut[l];
    for (int co = 0; co < co_n; co++) {
      double s = 0.0;
      for (int b = 0; b < B; b++)
        for (size_t c = 0; c < C; c++) s += g[((size_t)b * co_n + co) * C + c];
      gb[l][co] = (float)s;
    }
#pragma omp parallel for collapse(2) schedule(static)
    for (int co = 0; co < co_n; co++)
      for (int t = 0; t < 27; t++)
        for (int ci = 0; ci < ci_n; ci++) {
          double s = 0.0;
          for (int b = 0; b < B; b++)
            for (int zz = 0; zz < nz; zz++)
              for (int yy = 0; yy < ny; yy++)
                for (int xx = 0; xx < nx; xx++) {
                  const int qx = xx + t % 3 - 1, qy = yy + (t / 3) % 3 - 1, qz = zz + t / 9 - 1;
                  if (qx < 0 || qy < 0 || qz < 0 || qx >= nx || qy >= ny || qz >= nz) continue;
                  s += (double)g[((size_t)b * co_n + co) * C + S.at(xx, yy, zz)] *
                       a[l][((size_t)b * ci_n + ci) * C + S.at(qx, qy, qz)];
                }
          gw[l][((size_t)co * 27 + t) * ci_n + ci] = (float)s;
        }
    if (l == 0) break;
    // dL/da of layer l's input, then through the ReLU of layer l - 1
    std::vector<float> ga((size_t)B * ci_n * C, 0.f);
#pragma omp parallel for collapse(2) schedule(static)
    for (int b = 0; b < B; b++)
      for (int ci = 0; ci < ci_n; ci++)
        for (int zz = 0; zz < nz; zz++)
          for (int yy = 0; yy < ny; yy++)
            for (int xx = 0; xx < nx; xx++) {
              double s = 0.0;
              for (int t = 0; t < 27; t++) {
                // cells o whose tap t reads this cell: o = cell - off_t
                const int ox = xx - (t % 3 - 1), oy = yy - ((t / 3) % 3 - 1), oz = zz - (t / 9 - 1);
                if (ox < 0 || oy < 0 || oz < 0 || ox >= nx || oy >= ny || oz >= nz) continue;
                for (int co = 0; co < co_n; co++)
                  s += (double)wb[l][((size_t)co * 27 + t) * ci_n + ci] * g[((size_t)b * co_n + co) * C + S.at(ox, oy, oz)];
              }
              const size_t k = ((size_t)b * ci_n + ci) * C + S.at(xx, yy, zz);
              ga[k] = z[l - 1][k] > 0.f ? (float)s : 0.f;
            }
    g.swap(ga);
  }
  return loss;
}

}  // extern "C"
