// pbf_cell_sort_noalloc: the neighbour-search sort (cell hash, stable
// counting sort, cell ranges) for callers that cannot allocate device
// memory.
//
// Some callers cannot call cudaMalloc at the point where they need the
// sort: code that runs while a stream is being captured into a CUDA graph,
// plug-ins whose host application owns every device allocation through its
// own pool, or real-time paths where an allocation (and the device-wide
// synchronisation it may cause) is not allowed.  This entry point needs no
// handle and allocates nothing: its scratch (keys, slots, bucket scratch,
// cell counts and offsets) lives in one file-scope __device__ array of fixed
// size, which every GPU that loads the library holds until the process exits.
//
// Limits: n <= PBF_NOALLOC_MAX_PARTICLES particles and
// Gx*Gy*Gz <= PBF_NOALLOC_MAX_CELLS cells (7.3 MB of device memory).
//
// The first call on a device looks up the array's device address (with that
// device current) and caches it; make that first call before any stream
// capture.  All calls share the one array: calls whose work overlaps on the
// GPU (different streams, or different host threads on one device) race on it
// and must be serialised by the caller.  Each call clears the cell counts it
// uses before the histogram, so a call never sees the previous call's data.
#include <mutex>

#include "pbf103.h"
#include "pbf_internal.h"
#include "pbf_sort.cuh"

namespace pbf103 {
void set_last_error(const char *what, cudaError_t e);
}

namespace {

constexpr uint32_t kMaxN = PBF_NOALLOC_MAX_PARTICLES;
constexpr uint32_t kMaxC = PBF_NOALLOC_MAX_CELLS;
constexpr uint32_t kTile = 4096;                            // cells per scan tile
constexpr uint32_t kMaxTiles = (kMaxC + 1 + kTile - 1) / kTile;
// buckets of more than kRankMax entries are sorted by a block each
// (block_radix_stable); at most kMaxBig of them fit in kMaxN particles
constexpr uint32_t kRankMax = 4096;
constexpr uint32_t kMaxBig = kMaxN / (kRankMax + 1) + 1;
// words: keys, slots, tmp (n each); counts, offsets (C + 2 each); tile sums;
// the queue of large buckets (count, then cells)
constexpr size_t kWords = 3ull * kMaxN + 2ull * (kMaxC + 2) + kMaxTiles + 4 + 1 + kMaxBig;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kWords];

struct Scratch {
    uint32_t *keys, *slots, *tmp, *counts, *offsets, *tsum, *big;
};

Scratch carve(uint32_t *base)
{
    Scratch s;
    s.keys = base;
    s.slots = s.keys + kMaxN;
    s.tmp = s.slots + kMaxN;
    s.counts = s.tmp + kMaxN;
    s.offsets = s.counts + (kMaxC + 2);
    s.tsum = s.offsets + (kMaxC + 2);
    s.big = s.tsum + kMaxTiles + 4;
    return s;
}

// device address of the scratch array, per device, looked up once
std::mutex g_mu;
uint32_t *g_ptr[256];

__device__ __forceinline__ uint32_t hash_of(float x, float y, float z, float cw, uint3 g)
{
    const uint32_t gx = (uint32_t)__float2int_rd(__fdiv_rn(x, cw)) & (g.x - 1u);
    const uint32_t gy = (uint32_t)__float2int_rd(__fdiv_rn(y, cw)) & (g.y - 1u);
    const uint32_t gz = (uint32_t)__float2int_rd(__fdiv_rn(z, cw)) & (g.z - 1u);
    return gz * g.x * g.y + gy * g.x + gx;
}

__global__ void na_hash_count(const float *__restrict__ x, uint32_t n, float cw, uint3 g, Scratch s)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = hash_of(x[3 * i], x[3 * i + 1], x[3 * i + 2], cw, g);
    s.keys[i] = k;
    s.slots[i] = atomicAdd(s.counts + k, 1u);
}

__global__ void na_tile_sums(uint32_t C, Scratch s)
{
    __shared__ uint32_t part[256];
    const uint32_t t = blockIdx.x, base = t * kTile;
    uint32_t v = 0;
    for (uint32_t c = base + threadIdx.x; c < base + kTile && c < C; c += 256) v += s.counts[c];
    part[threadIdx.x] = v;
    __syncthreads();
    for (uint32_t o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) s.tsum[t] = part[0];
}

// one thread: exclusive scan of the (at most kMaxTiles) tile sums; empties
// the large-bucket queue that na_rank fills next
__global__ void na_tile_scan(uint32_t ntiles, uint32_t C, Scratch s)
{
    s.big[0] = 0;
    uint32_t run = 0;
    for (uint32_t t = 0; t < ntiles; ++t) {
        const uint32_t v = s.tsum[t];
        s.tsum[t] = run;
        run += v;
    }
    s.offsets[C] = run;
}

__global__ void na_scan_tiles(uint32_t C, Scratch s)
{
    __shared__ uint32_t buf[kTile];
    __shared__ uint32_t warp_tot[8];
    const uint32_t t = blockIdx.x, base = t * kTile;
    for (uint32_t c = threadIdx.x; c < kTile; c += 256) buf[c] = (base + c < C) ? s.counts[base + c] : 0u;
    __syncthreads();
    // each of the 256 threads scans 16 consecutive cells
    uint32_t loc[16], sum = 0;
    for (int k = 0; k < 16; ++k) {
        loc[k] = sum;
        sum += buf[threadIdx.x * 16 + k];
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t inc = sum;
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    uint32_t wpre = 0;
    for (uint32_t w = 0; w < warp; ++w) wpre += warp_tot[w];
    const uint32_t pre = s.tsum[t] + wpre + inc - sum;
    for (int k = 0; k < 16; ++k) {
        const uint32_t c = base + threadIdx.x * 16 + k;
        if (c < C) s.offsets[c] = pre + loc[k];
    }
}

__global__ void na_scatter(uint32_t n, Scratch s)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) s.tmp[s.offsets[s.keys[i]] + s.slots[i]] = i;
}

// stable position = bucket start + number of smaller indices in the bucket;
// a bucket above kRankMax entries is queued (by its member of atomic slot 0)
// for na_big instead
__global__ void na_rank(uint32_t n, Scratch s, uint32_t *__restrict__ perm)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = s.keys[i];
    const uint32_t st = s.offsets[k], en = s.offsets[k + 1];
    if (en - st > kRankMax) {
        if (s.slots[i] == 0) s.big[1 + atomicAdd(s.big, 1u)] = k;
        return;
    }
    uint32_t r = 0;
    for (uint32_t t = st; t < en; ++t) r += (s.tmp[t] < i) ? 1u : 0u;
    perm[st + r] = i;
}

// the queued large buckets, a block each: stable order by input index
__global__ void __launch_bounds__(pbf103::kRadixThreads) na_big(uint32_t n, Scratch s, uint32_t *__restrict__ perm)
{
    __shared__ pbf103::RadixSmem sm;
    __shared__ uint32_t base[16], tot[16];
    const uint32_t nb = s.big[0];
    for (uint32_t q = blockIdx.x; q < nb; q += gridDim.x) {
        const uint32_t k = s.big[1 + q];
        const uint32_t st = s.offsets[k], en = s.offsets[k + 1];
        pbf103::block_radix_stable(s.tmp + st, perm + st, en - st, 0xFFFFFFFFu, pbf103::radix_bits(n), sm, base,
                                   tot);
    }
}

__global__ void na_ranges(uint32_t C, Scratch s, uint32_t *__restrict__ cs, uint32_t *__restrict__ ce)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const uint32_t a = s.offsets[c], b = s.offsets[c + 1];
    cs[c] = (a == b) ? 0xFFFFFFFFu : a;
    ce[c] = (a == b) ? 0xFFFFFFFFu : b;
}

bool pow2(uint32_t v) { return v && !(v & (v - 1)); }

}  // namespace

extern "C" pbf_status pbf_cell_sort_noalloc(const float *x_dev, uint32_t n, float cell_width,
                                            const uint32_t grid[3], uint32_t *perm_dev, uint32_t *cell_start_dev,
                                            uint32_t *cell_end_dev, void *stream)
{
    if (!grid || !(cell_width > 0.f) || (n && (!x_dev || !perm_dev)) || !cell_start_dev || !cell_end_dev)
        return PBF_ERROR_INVALID_ARGUMENT;
    if (!pow2(grid[0]) || !pow2(grid[1]) || !pow2(grid[2])) return PBF_ERROR_INVALID_ARGUMENT;
    const uint64_t C64 = (uint64_t)grid[0] * grid[1] * grid[2];
    if (n > kMaxN || C64 > kMaxC) return PBF_ERROR_CAPACITY;  // beyond the fixed scratch
    const uint32_t C = (uint32_t)C64;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 256) {
        pbf103::set_last_error("cudaGetDevice", e);
        return PBF_ERROR_CUDA;
    }
    uint32_t *base;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_ptr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) {
                pbf103::set_last_error("cudaGetSymbolAddress", e);
                return PBF_ERROR_CUDA;
            }
            g_ptr[dev] = static_cast<uint32_t *>(p);
        }
        base = g_ptr[dev];
    }
    const Scratch s = carve(base);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint3 g = make_uint3(grid[0], grid[1], grid[2]);
    const uint32_t ntiles = (C + kTile - 1) / kTile;
    // the histogram must start from zero: clear this call's cells
    e = cudaMemsetAsync(s.counts, 0, 4ull * (C + 1), st);
    if (e != cudaSuccess) {
        pbf103::set_last_error("cudaMemsetAsync", e);
        return PBF_ERROR_CUDA;
    }
    if (n) na_hash_count<<<(n + 255) / 256, 256, 0, st>>>(x_dev, n, cell_width, g, s);
    na_tile_sums<<<ntiles, 256, 0, st>>>(C, s);
    na_tile_scan<<<1, 1, 0, st>>>(ntiles, C, s);
    na_scan_tiles<<<ntiles, 256, 0, st>>>(C, s);
    if (n) {
        na_scatter<<<(n + 255) / 256, 256, 0, st>>>(n, s);
        na_rank<<<(n + 255) / 256, 256, 0, st>>>(n, s, perm_dev);
        if (n > kRankMax) na_big<<<kMaxBig, pbf103::kRadixThreads, 0, st>>>(n, s, perm_dev);
    }
    na_ranges<<<(C + 255) / 256, 256, 0, st>>>(C, s, cell_start_dev, cell_end_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        pbf103::set_last_error("pbf_cell_sort_noalloc launch", e);
        return PBF_ERROR_CUDA;
    }
    return PBF_SUCCESS;
}
