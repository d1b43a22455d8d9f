// Shared device utilities: prefix sum, stable cell binning, error recording.
#include <climits>
#include <cstdio>
#include <cstring>

#include "spss_internal.cuh"

namespace spss
{

static thread_local char g_last_error[512];

void record_cuda_error(cudaError_t e, const char *what, const char *file, int line)
{
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
}

int check_launch(const char *what)
{
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
  {
    record_cuda_error(e, what, __FILE__, __LINE__);
    return SPSS_ERR_CUDA;
  }
  return SPSS_OK;
}

const char *last_error_text()
{
  return g_last_error;
}

// ------------------------------------------------------------------ scan

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Exclusive scan of one tile per block; block totals to `sums`.  When the
// whole input fits one tile the total is also written to out[n].
__global__ void scan_tile_kernel(const int *__restrict__ in, int *__restrict__ out, int *__restrict__ sums, int n)
{
  __shared__ int warp_tot[kScanThreads / 32];
  pdl_enter();
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int local = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; ++q)
  {
    v[q] = (base + q < n) ? in[base + q] : 0;
    local += v[q];
  }
  // inclusive scan of the per-thread totals across the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = local;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1)
  {
    int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0)
  {
    int w = (lane < kScanThreads / 32) ? warp_tot[lane] : 0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1)
    {
      int y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  int excl = x - local + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
  for (int q = 0; q < kScanItems; ++q)
  {
    if (base + q < n) out[base + q] = excl;
    excl += v[q];
  }
  if (threadIdx.x == kScanThreads - 1)
  {
    const int total = warp_tot[kScanThreads / 32 - 1];
    if (sums) sums[blockIdx.x] = total;
    if (gridDim.x == 1) out[n] = total;
  }
}

__global__ void scan_add_kernel(int *__restrict__ out, const int *__restrict__ block_off, int n, int nblocks)
{
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += block_off[i / kScanTile];
  if (i == 0) out[n] = block_off[nblocks];
}

int Scanner::run(const int *in, int *out, int n, cudaStream_t stream, unsigned long long &launches, bool chained)
{
  return run_level(in, out, n, 0, stream, launches, chained);
}

int Scanner::run_level(const int *in, int *out, int n, size_t level, cudaStream_t stream,
                       unsigned long long &launches, bool chained)
{
  if (n <= 0)
  {
    SPSS_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int), stream));
    return SPSS_OK;
  }
  const int nblocks = (n + kScanTile - 1) / kScanTile;
  if (nblocks == 1)
  {
    SPSS_CUDA_TRY(launch_chained(chained, scan_tile_kernel, 1, kScanThreads, 0, stream, in, out, (int *) nullptr, n));
    ++launches;
    return check_launch("scan_tile_kernel");
  }
  if (levels.size() < 2 * (level + 1)) levels.resize(2 * (level + 1));
  SPSS_TRY(levels[2 * level].reserve(nblocks));
  SPSS_TRY(levels[2 * level + 1].reserve(nblocks + 1));
  int *sums = levels[2 * level].ptr;       // device pointers stay valid if `levels` grows
  int *sums_off = levels[2 * level + 1].ptr;
  SPSS_CUDA_TRY(launch_chained(chained, scan_tile_kernel, nblocks, kScanThreads, 0, stream, in, out, sums, n));
  ++launches;
  SPSS_TRY(check_launch("scan_tile_kernel"));
  SPSS_TRY(run_level(sums, sums_off, nblocks, level + 1, stream, launches, chained));
  SPSS_CUDA_TRY(launch_chained(chained, scan_add_kernel, (n + 255) / 256, 256, 0, stream, out,
                               (const int *) sums_off, n, nblocks));
  ++launches;
  return check_launch("scan_add_kernel");
}

// ------------------------------------------------------------------ binning

__global__ void bin_count_kernel(const int *__restrict__ cell_of, int n, int *__restrict__ count,
                                 int *__restrict__ slot)
{
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) slot[i] = atomicAdd(&count[cell_of[i]], 1);
}

__global__ void bin_scatter_kernel(const int *__restrict__ cell_of, const int *__restrict__ slot,
                                   const int *__restrict__ offsets, int n, int *__restrict__ members)
{
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) members[offsets[cell_of[i]] + slot[i]] = i;
}

// Members of one cell into ascending order (cells hold a handful of particles):
// up to kSortRegs members are sorted in registers by an odd-even transposition
// network (all loads issued together, one store each), larger cells by an
// insertion sort in place.
constexpr int kSortRegs = 8;

__global__ void bin_sort_kernel(const int *__restrict__ offsets, int ncell, int *__restrict__ members)
{
  pdl_enter();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int b = offsets[c], e = offsets[c + 1];
  const int m = e - b;
  if (m <= 1) return;
  if (m <= kSortRegs)
  {
    int v[kSortRegs];
#pragma unroll
    for (int k = 0; k < kSortRegs; ++k) v[k] = k < m ? members[b + k] : INT_MAX;
#pragma unroll
    for (int r = 0; r < kSortRegs; ++r)
#pragma unroll
      for (int k = r & 1; k + 1 < kSortRegs; k += 2)
      {
        const int lo = min(v[k], v[k + 1]), hi = max(v[k], v[k + 1]);
        v[k] = lo;
        v[k + 1] = hi;
      }
#pragma unroll
    for (int k = 0; k < kSortRegs; ++k)
      if (k < m) members[b + k] = v[k];
    return;
  }
  for (int q = b + 1; q < e; ++q)
  {
    const int v = members[q];
    int r = q - 1;
    while (r >= b && members[r] > v)
    {
      members[r + 1] = members[r];
      --r;
    }
    members[r + 1] = v;
  }
}

int Binner::run(const int *cell_of, int n, int ncell_in, cudaStream_t stream, unsigned long long &launches,
                bool chained)
{
  ncell = ncell_in;
  SPSS_TRY(count.reserve(ncell));
  SPSS_TRY(offsets.reserve(ncell + 1));
  SPSS_TRY(slot.reserve(n));
  SPSS_TRY(members.reserve(n));
  SPSS_CUDA_TRY(cudaMemsetAsync(count.ptr, 0, sizeof(int) * ncell, stream));
  const int tb = 256;
  // the count follows a memset: an ordinary launch
  bin_count_kernel<<<(n + tb - 1) / tb, tb, 0, stream>>>(cell_of, n, count.ptr, slot.ptr);
  ++launches;
  SPSS_TRY(check_launch("bin_count_kernel"));
  SPSS_TRY(scanner.run(count.ptr, offsets.ptr, ncell, stream, launches, chained));
  SPSS_CUDA_TRY(launch_chained(chained, bin_scatter_kernel, (n + tb - 1) / tb, tb, 0, stream, cell_of,
                               (const int *) slot.ptr, (const int *) offsets.ptr, n, members.ptr));
  ++launches;
  SPSS_TRY(check_launch("bin_scatter_kernel"));
  SPSS_CUDA_TRY(launch_chained(chained, bin_sort_kernel, (ncell + tb - 1) / tb, tb, 0, stream,
                               (const int *) offsets.ptr, ncell, members.ptr));
  ++launches;
  return check_launch("bin_sort_kernel");
}

}  // namespace spss
