// leap_rotate_average_noalloc: the all-FP64 rotate + average stage for callers
// that cannot allocate device memory.  Its only scratch (the channel
// wavelength table and the per-slab partial sums) lives in one file-scope
// device array, so a call allocates nothing.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cudaTypedefs.h>

#include "leap_gb300.h"
#include "kernels_rotate.cuh"

using namespace leapgb;

// The scratch array.  Every GPU that loads the library holds it until exit;
// all calls on a device share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[LEAP_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;

// Per device: the scratch array's device address and the SM count, valid for the CUDA
// context they were looked up in.  A device reset or another context made current on
// the device loads the module again, at another address, so the entry is keyed by the
// context's unique ID (cuCtxGetId: IDs are never reused within a process).
struct DeviceSetup {
  unsigned long long ctx_id = 0;
  void* scratch = nullptr;
  int sms = 0;
};
std::mutex g_mutex;
DeviceSetup g_setup[kMaxDevices];

thread_local char g_err[256] = {0};  // fixed buffer: reporting an error allocates nothing either

int fail(int code, const char* msg) {
  std::strncpy(g_err, msg, sizeof(g_err) - 1);
  g_err[sizeof(g_err) - 1] = 0;
  return code;
}

template <typename Fn>
Fn driver_entry(const char* name, int version) {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &f, version, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<Fn>(f);
}

// Unique ID of the context current on this thread (0 if none can be read).
unsigned long long current_context_id() {
  static const auto get_current = driver_entry<PFN_cuCtxGetCurrent_v4000>("cuCtxGetCurrent", 4000);
  static const auto get_id = driver_entry<PFN_cuCtxGetId_v12000>("cuCtxGetId", 12000);
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Wavelengths of the channels, formed as the reference's
// Constants::GetChannelWavelength does: c / (f0 + ch*df), no fused multiply-add;
// then their rounded reciprocals (lam[channels + c]).
__global__ void fill_wavelengths(double* lam, int channels, double f0, double df) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < channels; c += gridDim.x * blockDim.x) {
    const double l = __ddiv_rn(kSpeedOfLight, __dadd_rn(f0, __dmul_rn(static_cast<double>(c), df)));
    lam[c] = l;
    lam[channels + c] = __drcp_rn(l);
  }
}

// Launches through cudaLaunchKernelEx, whose return value is this launch's own status:
// an error left over from the caller's earlier work is neither reported nor cleared.
template <typename... Params, typename... Args>
cudaError_t launch_kernel(void (*kernel)(Params...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <typename VisT, int P>
cudaError_t launch_rotate(const RotateArgs& a, dim3 grid, cudaStream_t s) {
  return launch_kernel(rotate_average_fp64<VisT, P, 2, true>, grid, dim3(128), s, a);
}

}  // namespace

extern "C" const char* leap_noalloc_last_error(void) { return g_err; }

extern "C" int32_t leap_rotate_average_noalloc(int32_t vis_type, const void* vis, const double* uvw, int64_t rows,
                                               int32_t channels, int32_t pols, int32_t nbl, double freq_start_hz,
                                               double freq_inc_hz, const double* dd, int32_t ndirections,
                                               double* avg_out, void* stream) {
  if (!vis || !uvw || !dd || !avg_out) return fail(LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (vis_type != LEAP_VIS_C64 && vis_type != LEAP_VIS_C128) return fail(LEAP_ERR_INVALID_ARGUMENT, "unknown vis type");
  if (pols != 1 && pols != 2 && pols != 4) return fail(LEAP_ERR_INVALID_ARGUMENT, "pols must be 1, 2 or 4");
  if (rows <= 0 || channels <= 0 || nbl <= 0 || ndirections <= 0)
    return fail(LEAP_ERR_INVALID_ARGUMENT, "empty integration or no directions");
  if (rows % nbl != 0) return fail(LEAP_ERR_INVALID_ARGUMENT, "rows not a multiple of the baseline count");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(LEAP_ERR_CUDA, "no current CUDA device");
  if (dev < 0 || dev >= kMaxDevices) return fail(LEAP_ERR_INVALID_ARGUMENT, "device index beyond the set-up table");

  // Set-up, once per device (and again if the device's context changed), with that
  // device current: the host-side name of the array is not a device address, so ask
  // the runtime for it.
  unsigned char* scratch = nullptr;
  int sms = 0;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    DeviceSetup& st = g_setup[dev];
    const unsigned long long id = current_context_id();
    if (!st.scratch || id == 0 || id != st.ctx_id) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) return fail(LEAP_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
      int n = 0;
      if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
        return fail(LEAP_ERR_CUDA, "cannot read the device's multiprocessor count");
      st.scratch = p;
      st.sms = n;
      st.ctx_id = current_context_id();
    }
    scratch = static_cast<unsigned char*>(st.scratch);
    sms = st.sms;
  }

  // Scratch layout: [wavelengths, reciprocals, 256-byte aligned][slab partial sums].
  const size_t lam_bytes = ((2 * sizeof(double) * static_cast<size_t>(channels) + 255) / 256) * 256;
  if (lam_bytes > LEAP_NOALLOC_SCRATCH_BYTES)
    return fail(LEAP_ERR_INVALID_ARGUMENT, "channel count exceeds the no-allocation scratch limit");
  const size_t avail = LEAP_NOALLOC_SCRATCH_BYTES - lam_bytes;
  const int T = static_cast<int>(rows / nbl);
  const int tiles = (nbl + 31) / 32;
  const int dgroups = (ndirections + 7) / 8;  // 4 warps x 2 directions per block
  const size_t slab_bytes = sizeof(double2) * static_cast<size_t>(ndirections) * pols * nbl;
  // Timestep slabs: about 8 blocks per SM, as many as fit in the scratch.
  int nts = static_cast<int>(std::min<int64_t>(T, std::max<int64_t>(1, (int64_t(sms) * 8 + int64_t(tiles) * dgroups - 1) /
                                                                           (int64_t(tiles) * dgroups))));
  while (nts > 1 && slab_bytes * nts > avail) --nts;
  const int t_per = (T + nts - 1) / nts;
  nts = (T + t_per - 1) / t_per;

  RotateArgs a{};
  a.vis = vis;
  a.uvw = uvw;
  a.dd = dd;
  a.lambda = reinterpret_cast<const double*>(scratch);
  a.inv_lambda = reinterpret_cast<const double*>(scratch) + channels;
  a.rows = rows;
  a.channels = channels;
  a.pols = pols;
  a.nbl = nbl;
  a.timesteps = T;
  a.ndir = ndirections;
  a.f0 = freq_start_hz;
  a.df = freq_inc_hz;
  a.t_per_slab = t_per;
  a.c_per_slab = channels;
  a.n_tslab = nts;
  a.n_cslab = 1;
  a.out = nts > 1 ? reinterpret_cast<double2*>(scratch + lam_bytes) : reinterpret_cast<double2*>(avg_out);

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = launch_kernel(fill_wavelengths, dim3((channels + 255) / 256), dim3(256), s,
                                reinterpret_cast<double*>(scratch), channels, freq_start_hz, freq_inc_hz);
  if (e != cudaSuccess) return fail(LEAP_ERR_CUDA, cudaGetErrorString(e));
  const dim3 grid(tiles, dgroups, nts);
  if (vis_type == LEAP_VIS_C64) {
    if (pols == 1) e = launch_rotate<float2, 1>(a, grid, s);
    else if (pols == 2) e = launch_rotate<float2, 2>(a, grid, s);
    else e = launch_rotate<float2, 4>(a, grid, s);
  } else {
    if (pols == 1) e = launch_rotate<double2, 1>(a, grid, s);
    else if (pols == 2) e = launch_rotate<double2, 2>(a, grid, s);
    else e = launch_rotate<double2, 4>(a, grid, s);
  }
  if (e != cudaSuccess) return fail(LEAP_ERR_CUDA, cudaGetErrorString(e));
  if (nts > 1) {
    const int64_t n = static_cast<int64_t>(ndirections) * pols * nbl;
    const int blocks = static_cast<int>(std::min<int64_t>((n + 255) / 256, int64_t(sms) * 32));
    e = launch_kernel(reduce_slabs, dim3(blocks), dim3(256), s, reinterpret_cast<const double2*>(scratch + lam_bytes),
                      nts, n, reinterpret_cast<double2*>(avg_out));
    if (e != cudaSuccess) return fail(LEAP_ERR_CUDA, cudaGetErrorString(e));
  }
  return LEAP_OK;
}
