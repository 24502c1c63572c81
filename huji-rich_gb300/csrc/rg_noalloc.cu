// rg_noalloc.cu -- SimpleCFL time step for callers that must not allocate
// device memory.
//
// Some hosts own every byte of GPU memory through their own allocator: a
// multi-physics driver that hands RICH's hydro step a fixed arena, or a
// framework whose caching pool is the only thing allowed to call
// cudaMalloc / cudaFree (those calls synchronise the whole device and bypass
// the pool's accounting).  Such a caller cannot create an rg_handle, which
// allocates its mesh, state and status buffers.  rg_cfl_dt_noalloc computes
// the same dt as rg_cfl_dt from caller-owned device arrays and allocates
// nothing: the only memory it needs beyond its inputs and its output -- the
// per-block minima of the reduction and a completion counter -- lives in the
// file-scope array below, which every GPU that loads the library holds
// until the process exits.
//
// The array is shared by every call on a device and keeps the last call's
// contents; each call clears the completion counter before its kernel runs
// (the per-block minima are always written before they are read).  Calls
// that overlap on the GPU (two streams, or two host threads) race on the
// array: serialise them.  The first call on each device looks up the array's
// device address (cudaGetSymbolAddress) with that device current.  Under the
// CUDA runtime's lazy module loading (its default) that lookup is also when
// the driver loads this library's device code and creates the array, which
// takes driver memory and can block the device once: make the first call
// during set-up, before the caller's allocator takes over and before any
// stream capture.
//
// The caller's pointers are checked before anything is enqueued: each must
// be device (or managed) memory of the current device, `cells` and
// `edge_velocities` 16-byte aligned (the kernel reads them as double2), the
// others naturally aligned.  Indices are not checked: a cell_faces entry
// outside the edge_velocities array is read out of bounds.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "rg_div.cuh"
#include "rg_internal.cuh"

namespace {

constexpr int kBlock = 256;
// 4096 blocks of 256 threads: at most 1,048,576 cells per call
constexpr int kMaxBlocks = 4096;
constexpr long long kMaxCells = static_cast<long long>(kMaxBlocks) * kBlock;
constexpr int kMaxDevices = 64;

// [0, kMaxBlocks): per-block minima (bit patterns of positive doubles);
// [kMaxBlocks]: completion counter.  32 KiB + 256 B.
static __device__ __align__(256) unsigned long long g_cfl_scratch[kMaxBlocks + 32];

std::mutex g_setup_mutex;
unsigned long long* g_scratch_dev[kMaxDevices] = {};

// Device address of g_cfl_scratch on the current device (looked up once per
// device; in host code the symbol itself is only a stand-in).
cudaError_t scratch_address(int device, unsigned long long** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_dev[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_cfl_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_dev[device] = static_cast<unsigned long long*>(p);
  }
  *out = g_scratch_dev[device];
  return cudaSuccess;
}

// simple_cfl.cpp:28-47 per cell (radius = VoronoiMesh::GetWidth,
// VoronoiMesh.cpp:410-413), then the min of simple_cfl.cpp:64 / lazy_min
// through the scratch array; the last block writes cfl * min.
__global__ void __launch_bounds__(kBlock)
    k_cfl_noalloc(int n, const double* __restrict__ cells, const double* __restrict__ volume,
                  const int* __restrict__ off, const int* __restrict__ faces, const double* __restrict__ ev,
                  double gamma, double cfl, unsigned long long* scratch, double* dt_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double x = __longlong_as_double(static_cast<long long>(rg::kInfBits));
  if (i < n) {
    const double2 dp = reinterpret_cast<const double2*>(cells)[2 * i];
    const double2 uv = reinterpret_cast<const double2*>(cells)[2 * i + 1];
    const double radius = rg::root(rg::quot(volume[i], rg::kPi));
    const double cs = rg::root(rg::quot(gamma * dp.y, dp.x));
    double res = 0;
    for (int k = off[i]; k < off[i + 1]; ++k) {
      const double2 w = reinterpret_cast<const double2*>(ev)[faces[k]];
      const double dx = uv.x - w.x, dy = uv.y - w.y;
      res = fmax(res, rg::quot(cs + rg::root(dx * dx + dy * dy), radius));
    }
    x = rg::quot(1.0, res);
  }
  unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x));
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = ob < bits ? ob : bits;
  }
  __shared__ unsigned long long wmin[kBlock / 32];
  __shared__ bool last;
  if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long bm = wmin[0];
    for (int w = 1; w < kBlock / 32; ++w) bm = wmin[w] < bm ? wmin[w] : bm;
    scratch[blockIdx.x] = bm;
    __threadfence();
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kMaxBlocks);
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    unsigned long long m = rg::kInfBits;
    for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += kBlock) {
      const unsigned long long v = *reinterpret_cast<volatile unsigned long long*>(scratch + b);
      m = v < m ? v : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, m, o);
      m = ob < m ? ob : m;
    }
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long bm = wmin[0];
      for (int w = 1; w < kBlock / 32; ++w) bm = wmin[w] < bm ? wmin[w] : bm;
      *dt_out = cfl * __longlong_as_double(static_cast<long long>(bm));
    }
  }
}

bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

// True when p is device or managed memory that `device` can address (a host
// pointer, pinned or not, would fault the kernel or read the wrong memory).
bool on_device(const void* p, int device) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeDevice) return a.device == device;
  return a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" rg_status rg_cfl_dt_noalloc(int32_t n_cells, const double* cells, const double* volume,
                                       const int32_t* cell_face_offset, const int32_t* cell_faces,
                                       const double* edge_velocities, double gamma, double cfl,
                                       double* dt_out, void* stream) {
  if (n_cells <= 0 || n_cells > kMaxCells) return RG_ERR_INVALID_ARGUMENT;
  if (!cells || !volume || !cell_face_offset || !cell_faces || !edge_velocities || !dt_out)
    return RG_ERR_INVALID_ARGUMENT;
  // double2 loads need 16-byte alignment; the scalar arrays their own size
  if (!aligned(cells, 16) || !aligned(edge_velocities, 16) || !aligned(volume, 8) || !aligned(dt_out, 8) ||
      !aligned(cell_face_offset, 4) || !aligned(cell_faces, 4))
    return RG_ERR_INVALID_ARGUMENT;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
    cudaGetLastError();
    return RG_ERR_CUDA;
  }
  const void* ptrs[] = {cells, volume, cell_face_offset, cell_faces, edge_velocities, dt_out};
  for (const void* p : ptrs)
    if (!on_device(p, device)) return RG_ERR_INVALID_ARGUMENT;
  unsigned long long* scratch = nullptr;
  if (scratch_address(device, &scratch) != cudaSuccess) {
    cudaGetLastError();
    return RG_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the completion counter must start at zero; the minima are overwritten
  if (cudaMemsetAsync(scratch + kMaxBlocks, 0, sizeof(unsigned long long), s) != cudaSuccess) {
    cudaGetLastError();
    return RG_ERR_CUDA;
  }
  const int blocks = (n_cells + kBlock - 1) / kBlock;
  k_cfl_noalloc<<<blocks, kBlock, 0, s>>>(n_cells, cells, volume, cell_face_offset, cell_faces,
                                           edge_velocities, gamma, cfl, scratch, dt_out);
  if (cudaGetLastError() != cudaSuccess) return RG_ERR_CUDA;
  return RG_OK;
}
