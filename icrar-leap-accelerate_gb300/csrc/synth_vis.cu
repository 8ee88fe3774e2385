// Device generator of the synthetic point-source visibilities (leap_synth.h).
// One thread per (channel, row) sample group writes its `pols` complex<float>
// values; the model phase is formed and reduced in FP64.  Noise: a
// splitmix64-style mix of (seed, element index) gives two 53-bit uniforms per
// element, turned into a normal pair by the Box-Muller transform.
#include <cuda_runtime.h>
#include <stdint.h>

#include "leap_synth.h"

namespace {

constexpr double kSpeedOfLight = 299792458.0;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double unit_open(uint64_t bits) {  // (0, 1]
  return (static_cast<double>(bits >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

__global__ void synth_fill(float2* __restrict__ vis, const double* __restrict__ delay, const double2* __restrict__ gg,
                           int64_t rows, int nbl, int channels, int pols, double f0, double df, double scale,
                           uint64_t seed) {
  const int64_t groups = rows * channels;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < groups;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i % rows;
    const int c = static_cast<int>(i / rows);
    const double nu = f0 + c * df;
    // turns = delay * nu / c, reduced to [-0.5, 0.5) before the sine
    double turns = delay[r] * (nu / kSpeedOfLight);
    turns -= rint(turns);
    double s, co;
    sincospi(2.0 * turns, &s, &co);
    const double2 g = gg[r % nbl];
    const double mre = g.x * co - g.y * s, mim = g.x * s + g.y * co;
    for (int p = 0; p < pols; ++p) {
      const uint64_t idx = static_cast<uint64_t>(i) * pols + p;
      double nre = 0.0, nim = 0.0;
      if (scale > 0.0) {
        const uint64_t h1 = mix64(seed * 0x9e3779b97f4a7c15ull + 2 * idx + 1);
        const uint64_t h2 = mix64(h1 ^ (0xd1b54a32d192ed03ull + 2 * idx));
        const double rad = sqrt(-2.0 * log(unit_open(h1)));
        double sn, cs;
        sincospi(2.0 * unit_open(h2), &sn, &cs);
        nre = scale * rad * cs;
        nim = scale * rad * sn;
      }
      vis[i * pols + p] = make_float2(static_cast<float>(mre + nre), static_cast<float>(mim + nim));
    }
  }
}

}  // namespace

extern "C" int32_t leap_synth_fill_c64(void* vis, const double* delay, const double* gg, int64_t rows, int32_t nbl,
                                       int32_t channels, int32_t pols, double f0, double df, double sigma,
                                       uint64_t seed, void* stream) {
  if (!vis || !delay || !gg || rows <= 0 || nbl <= 0 || channels <= 0 || pols <= 0) return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t groups = rows * channels;
  const int64_t want = (groups + 255) / 256;
  const int grid = static_cast<int>(want < static_cast<int64_t>(sms) * 16 ? want : static_cast<int64_t>(sms) * 16);
  synth_fill<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<float2*>(vis), delay, reinterpret_cast<const double2*>(gg), rows, nbl, channels, pols, f0, df,
      sigma / 1.4142135623730951, seed);
  return static_cast<int32_t>(cudaGetLastError());
}
