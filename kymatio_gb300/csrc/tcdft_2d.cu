// DFT-GEMM tensor-core variants of the childless cascade tasks and the
// per-device DFT operand images they copy into shared memory.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "tcdft.cuh"

namespace kym {
namespace {

// float -> bf16 bits, round to nearest even (finite inputs).
uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float bf16_value(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
size_t kmajor_offset_host(int r, int k, int kp) {
  return (size_t)(r >> 3) * (kp >> 3) * 128 + (size_t)(k >> 3) * 128 + (size_t)(r & 7) * 16 + (size_t)(k & 7) * 2;
}

// Wop = [[Re W, -Im W], [Im W, Re W]] for W[v][y] = exp(+2 pi i v y / m),
// rows n (output, [Re | Im] halves of MP), K = [Re | Im] halves of MP, in
// the K-major core-matrix layout: the hi image, then the lo image.
std::vector<unsigned char> build_image(int m) {
  const int mp = (m + 7) / 8 * 8, kp = 2 * mp, np = 2 * mp;
  const size_t half = (size_t)np * kp * 2;
  std::vector<unsigned char> img(2 * half, 0);
  const double two_pi = 6.283185307179586476925286766559;
  for (int n = 0; n < np; ++n)
    for (int k = 0; k < kp; ++k) {
      const int y = n % mp, v = k % mp;
      double w = 0.0;
      if (y < m && v < m) {
        const double ang = two_pi * (double)(((long long)v * y) % m) / (double)m;
        const double c = std::cos(ang), s = std::sin(ang);
        const bool re_out = n < mp, re_in = k < mp;
        w = re_out ? (re_in ? c : -s) : (re_in ? s : c);
      }
      const uint16_t h = bf16_bits((float)w);
      const uint16_t l = bf16_bits((float)(w - (double)bf16_value(h)));
      const size_t off = kmajor_offset_host(n, k, kp);
      std::memcpy(img.data() + off, &h, 2);
      std::memcpy(img.data() + half + off, &l, 2);
    }
  return img;
}

std::mutex& image_mu() {
  static std::mutex m;
  return m;
}
std::map<std::pair<int, int>, void*>& images() {
  static std::map<std::pair<int, int>, void*> t;
  return t;
}

}  // namespace

const unsigned char* dft_operand_image(int m, size_t bytes) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(image_mu());
  auto key = std::make_pair(dev, m);
  auto it = images().find(key);
  if (it != images().end()) return static_cast<const unsigned char*>(it->second);
  const std::vector<unsigned char> img = build_image(m);
  if (img.size() != bytes) return nullptr;
  void* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
  if (cudaMemcpy(d, img.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(d);
    return nullptr;
  }
  images()[key] = d;
  return static_cast<const unsigned char*>(d);
}

}  // namespace kym

// 256x256 at J=3: the 68x68 childless groups (order 2 at (0,2) and (1,2),
// order 1 at j1=2), output 32x32.
KYM_TCDFT_VARIANT(68, 32, 4, 512)
KYM_TCDFT_VARIANT(68, 32, 2, 512)
