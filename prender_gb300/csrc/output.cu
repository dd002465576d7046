// 8-bit output of a rendered image (Render::OutputBmp, render.h:1563-1589,
// with ppm.h:22-27's to_int): per channel int(pow(clamp(x, 0, 1), g) * 255
// + 0.5) with g = 1/2.2, or g = gamma_offset when |gamma_offset| > 0.01
// (the reference then uses the offset itself as the exponent), written in
// the bitmap's cell(i, j) order: row i holds image row H - 1 - i; and the
// Radiance RGBE pixels of Render::OutputHdr.
#include <cuda_runtime.h>

#include <cstdint>

namespace pr {

__global__ void __launch_bounds__(256) to_rgb8_kernel(const float* __restrict__ rgb, int width, int height, double g,
                                                     uint8_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)width * height;
  if (i >= n) return;
  const int row = (int)(i / width), col = (int)(i % width);
  const int64_t src = (int64_t)(height - row - 1) * width + col;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double x = (double)rgb[3 * src + k];
    if (x < 0.0) x = 0.0;
    if (x > 1.0) x = 1.0;
    const int v = (int)(pow(x, g) * 255 + 0.5);
    out[3 * i + k] = (uint8_t)v;  // 0..255 for x in [0, 1]
  }
}

cudaError_t launch_to_rgb8(const float* rgb, int width, int height, double gamma_offset, uint8_t* out,
                           cudaStream_t stream) {
  const double g = (gamma_offset > 0.01 || gamma_offset < -0.01) ? gamma_offset : 0.4545454545454545454545;
  const int64_t n = (int64_t)width * height;
  if (n <= 0) return cudaSuccess;
  to_rgb8_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(rgb, width, height, g, out);
  return cudaGetLastError();
}

// Radiance RGBE pixels of an image for Render::OutputHdr (render.h:1649-1667,
// HDRImage::HDRPixel, hdr.h:30-44): d = max(r, g, b) in double; 0 when
// d <= 1e-32; else m 2^e = d (frexp), each channel (unsigned char)(c m 256 /
// d) and e + 128.  File scanline r holds image row r of pr_render's order
// (OutputHdr flips the rows once, HDRImage::save back again).
__global__ void __launch_bounds__(256) to_rgbe_kernel(const float* __restrict__ rgb, int64_t n,
                                                     uint8_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double r = fmax((double)rgb[3 * i], 0.0), g = fmax((double)rgb[3 * i + 1], 0.0),
               b = fmax((double)rgb[3 * i + 2], 0.0);
  double d = fmax(r, fmax(g, b));
  uchar4 q = make_uchar4(0, 0, 0, 0);
  if (d > 1e-32) {
    int e;
    const double m = frexp(d, &e);
    d = m * 256.0 / d;
    q = make_uchar4((unsigned char)(r * d), (unsigned char)(g * d), (unsigned char)(b * d), (unsigned char)(e + 128));
  }
  reinterpret_cast<uchar4*>(out)[i] = q;
}

cudaError_t launch_to_rgbe(const float* rgb, int width, int height, uint8_t* out, cudaStream_t stream) {
  const int64_t n = (int64_t)width * height;
  if (n <= 0) return cudaSuccess;
  to_rgbe_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(rgb, n, out);
  return cudaGetLastError();
}

}  // namespace pr
