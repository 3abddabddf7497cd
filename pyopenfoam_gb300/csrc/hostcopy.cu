// Host <-> device copies driven by the SMs: loads (stores) of page-locked
// host memory over NVLink-C2C, in place of the copy engines.
//
// On GB300 (Grace + Blackwell) page-locked host memory is addressable from
// the device, so a kernel can move it with ordinary 16-byte loads and
// stores.  Measured on GB300, four arrays of 1.07 GB in all (the 256^3
// system's diag, lower, upper and right-hand side): the kernel copies them
// in 5.1 ms every time (210 GB/s, the link's rate), while copy-engine copies
// of the same arrays in the same process took anywhere from 5.1 to 66 ms,
// step to step, with the GPU otherwise idle and no throttle reason active.
//
// Only memory that CUDA reports as page-locked host memory is read or
// written here (cudaPointerGetAttributes); anything else is refused with
// GBF_ERR_ARG, and the caller copies it another way.
#include "common.cuh"

namespace gbf {

// dst[i] = src[i] for i < n; four loads in flight per thread.
template <typename T>
__global__ void __launch_bounds__(256)
    host_copy_kernel(const T* __restrict__ src, T* __restrict__ dst, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    const T a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n; i += stride) dst[i] = src[i];
}

template <typename T>
static cudaError_t launch_copy(const void* src, void* dst, size_t bytes, int sms,
                               cudaStream_t s) {
  const long long n = (long long)(bytes / sizeof(T));
  if (n == 0) return cudaSuccess;
  // 16 blocks of 256 threads per SM: the link's rate (4 per SM measured
  // 2.8x slower on the same arrays)
  long long blocks = (n + 255) / 256;
  if (blocks > 16LL * sms) blocks = 16LL * sms;
  host_copy_kernel<T><<<(int)blocks, 256, 0, s>>>(static_cast<const T*>(src),
                                                  static_cast<T*>(dst), n);
  return cudaGetLastError();
}

// Body in the widest word both pointers are aligned to, the remaining bytes
// (fewer than one word) one by one.
static cudaError_t sm_copy(const void* src, void* dst, size_t bytes, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const uintptr_t a = (uintptr_t)src | (uintptr_t)dst;
  size_t g = 16;
  while (g > 1 && (a % g) != 0) g >>= 1;
  const size_t body = bytes / g * g;
  switch (g) {
    case 16: e = launch_copy<uint4>(src, dst, body, sms, s); break;
    case 8: e = launch_copy<uint2>(src, dst, body, sms, s); break;
    case 4: e = launch_copy<uint32_t>(src, dst, body, sms, s); break;
    case 2: e = launch_copy<uint16_t>(src, dst, body, sms, s); break;
    default: e = launch_copy<uint8_t>(src, dst, body, sms, s); break;
  }
  if (e == cudaSuccess && body < bytes)
    e = launch_copy<uint8_t>(static_cast<const char*>(src) + body,
                             static_cast<char*>(dst) + body, bytes - body, sms, s);
  return e;
}

// The device address of page-locked host memory at p, or nullptr when p is
// not page-locked host memory.
static const void* locked_host_address(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();  // an unregistered pointer may leave an error behind
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
  return at.devicePointer;
}

static bool is_device_memory(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace gbf

using namespace gbf;

extern "C" int gbf_copy_from_host(void* dst, const void* src_host, size_t bytes, void* stream) {
  if (bytes == 0) return GBF_OK;
  GBF_REQUIRE(dst && src_host, "copy_from_host: NULL pointer");
  const void* src = locked_host_address(src_host);
  GBF_REQUIRE(src, "copy_from_host: the source is not page-locked host memory");
  GBF_REQUIRE(is_device_memory(dst), "copy_from_host: the destination is not device memory");
  GBF_CHECK_CUDA(sm_copy(src, dst, bytes, as_stream(stream)));
  return GBF_OK;
}

extern "C" int gbf_copy_to_host(void* dst_host, const void* src, size_t bytes, void* stream) {
  if (bytes == 0) return GBF_OK;
  GBF_REQUIRE(dst_host && src, "copy_to_host: NULL pointer");
  const void* dst = locked_host_address(dst_host);
  GBF_REQUIRE(dst, "copy_to_host: the destination is not page-locked host memory");
  GBF_REQUIRE(is_device_memory(src), "copy_to_host: the source is not device memory");
  GBF_CHECK_CUDA(sm_copy(src, const_cast<void*>(dst), bytes, as_stream(stream)));
  return GBF_OK;
}
