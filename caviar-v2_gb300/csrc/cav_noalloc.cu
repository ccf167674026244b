// cav_noalloc.cu -- kinetic energy and temperature of caller-owned device arrays,
// with no device allocation by this library.
//
// Some callers cannot call cudaMalloc: code that runs while a stream is being
// captured into a CUDA graph (an allocation there invalidates the capture),
// code whose device memory belongs to another allocator (a framework's caching
// pool, a fixed arena carved out at start-up), and real-time loops in which the
// implicit synchronisation of cudaMalloc/cudaFree is not acceptable.  This entry
// point computes the same KE and T as the per-context reduction behind
// cavgpu_thermo (two passes, fixed order), but keeps its per-block partial sums
// in a file-scope __device__ array instead of allocating them.
#include <cuda_runtime.h>

#include <mutex>

#include "cav_common.cuh"

namespace {

constexpr int NA_BLOCK = 256;
constexpr int NA_ATOMS_PER_THREAD = 8;
constexpr int NA_MAX_BLOCKS = 8192;
constexpr int NA_SUMS = 5;  // sum m v^2, sum m v (3), sum m
// largest system: 8192 blocks x 256 threads x 8 atoms = 16,777,216 atoms
constexpr long long NA_MAX_ATOMS = (long long)NA_MAX_BLOCKS * NA_BLOCK * NA_ATOMS_PER_THREAD;

// 8192 x 5 doubles = 320 KiB on every device that loads the library, until exit.
// Every call overwrites exactly the slots it later reads, so nothing has to be
// cleared between calls; calls that overlap on the GPU share these slots and race.
static __device__ __align__(256) double g_ke_scratch[NA_MAX_BLOCKS * NA_SUMS];

struct KeArgs {
  double mass[CAVGPU_MAX_TYPES];
  int ntypes;
  long long n;
  int n_r_df;
  double k_b;
};

__global__ void __launch_bounds__(NA_BLOCK) k_ke_partials(const double *vel3, const uint64_t *type, KeArgs a,
                                                          double *scratch) {
  double s[NA_SUMS] = {0, 0, 0, 0, 0};
  const long long base = (long long)blockIdx.x * NA_BLOCK * NA_ATOMS_PER_THREAD;
#pragma unroll
  for (int k = 0; k < NA_ATOMS_PER_THREAD; ++k) {
    const long long i = base + (long long)k * NA_BLOCK + threadIdx.x;
    if (i < a.n) {
      const uint64_t t = type[i];
      const double m = t < (uint64_t)a.ntypes ? a.mass[t] : 0.0;  // unknown types contribute nothing
      const double vx = vel3[3 * i], vy = vel3[3 * i + 1], vz = vel3[3 * i + 2];
      s[0] += m * (vx * vx + vy * vy + vz * vz);
      s[1] += m * vx; s[2] += m * vy; s[3] += m * vz;
      s[4] += m;
    }
  }
  __shared__ double sh[NA_BLOCK / 32][NA_SUMS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NA_SUMS; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
  if (lane == 0)
    for (int q = 0; q < NA_SUMS; ++q) sh[wid][q] = s[q];
  __syncthreads();
  if (threadIdx.x < NA_SUMS) {
    double t = 0.0;
    for (int w = 0; w < NA_BLOCK / 32; ++w) t += sh[w][threadIdx.x];
    scratch[(size_t)blockIdx.x * NA_SUMS + threadIdx.x] = t;
  }
}

// out2 = {KE, T} as Atom_data::kinetic_energy_mpi_domain / finalize_temperature_mpi_domain
// (src/atom_data/kinetic_energy.cpp:26-134, 189-198) for n_r_df 0..3.
__global__ void __launch_bounds__(NA_BLOCK) k_ke_final(const double *scratch, int nblocks, KeArgs a, double *out2) {
  double s[NA_SUMS] = {0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += NA_BLOCK)
    for (int q = 0; q < NA_SUMS; ++q) s[q] += scratch[(size_t)b * NA_SUMS + q];
  __shared__ double sh[NA_BLOCK / 32][NA_SUMS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NA_SUMS; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
  if (lane == 0)
    for (int q = 0; q < NA_SUMS; ++q) sh[wid][q] = s[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[NA_SUMS];
    for (int q = 0; q < NA_SUMS; ++q) {
      t[q] = 0.0;
      for (int w = 0; w < NA_BLOCK / 32; ++w) t[q] += sh[w][q];
    }
    double ke2 = t[0];
    if (a.n_r_df >= 1 && a.n_r_df <= 3 && t[4] > 0) ke2 -= (t[1] * t[1] + t[2] * t[2] + t[3] * t[3]) / t[4];
    const double ke = 0.5 * ke2;
    const long long dof = 3 * a.n - a.n_r_df;
    out2[0] = ke;
    out2[1] = 2.0 * ke / (a.k_b * (double)dof);
  }
}

std::mutex g_init_mutex;
double *g_scratch_addr[256] = {nullptr};

// Device address of g_ke_scratch on the current device, looked up once per device.
// In host code the symbol is a host-side stand-in, not a device address.
int scratch_for_current_device(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
    cudaGetLastError();
    return CAVGPU_E_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_init_mutex);
  if (!g_scratch_addr[dev]) {
    double *p = nullptr;
    if (cudaGetSymbolAddress((void **)&p, g_ke_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return CAVGPU_E_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return CAVGPU_OK;
}

}  // namespace

extern "C" int cavgpu_kinetic_energy_noalloc(int64_t n, const double *vel3, const uint64_t *type, const double *mass,
                                             int32_t ntypes, int32_t n_r_df, double k_b, double *out2,
                                             void *stream) {
  if (n < 1 || !vel3 || !type || !mass || !out2 || ntypes < 1 || ntypes > CAVGPU_MAX_TYPES || n_r_df < 0 ||
      n_r_df > 3 || !(k_b > 0.0))
    return CAVGPU_E_ARG;
  if (n > NA_MAX_ATOMS) return CAVGPU_E_RANGE;
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  KeArgs a;
  for (int t = 0; t < CAVGPU_MAX_TYPES; ++t) a.mass[t] = t < ntypes ? mass[t] : 0.0;
  a.ntypes = ntypes;
  a.n = n;
  a.n_r_df = n_r_df;
  a.k_b = k_b;
  const int nblocks = (int)((n + (long long)NA_BLOCK * NA_ATOMS_PER_THREAD - 1) / ((long long)NA_BLOCK * NA_ATOMS_PER_THREAD));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_ke_partials<<<nblocks, NA_BLOCK, 0, st>>>(vel3, type, a, scratch);
  k_ke_final<<<1, NA_BLOCK, 0, st>>>(scratch, nblocks, a, out2);
  return cudaPeekAtLastError() == cudaSuccess ? CAVGPU_OK : CAVGPU_E_CUDA;
}
