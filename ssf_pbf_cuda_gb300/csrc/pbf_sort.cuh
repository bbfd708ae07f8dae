// Stable order of one large cell bucket, by one block of kRadixThreads
// threads: the bucket's entries (input index in the bits of imask, other
// bits ignored) sorted by ascending input index, which is the order a
// stable sort by cell gives (cub::DeviceRadixSort::SortPairs in the
// reference's USE_CUB path, src/pbf/interaction/cuda/pbf_neighbor_search_util.cu:177-198).
//
// LSD radix sort over the index bits, 4 bits a pass, in global memory: each
// pass is a digit histogram of the bucket, then chunks of kRadixChunk
// entries in order, each thread holding kRadixItems consecutive entries;
// an entry's place is its digit's start + the entries of that digit in
// earlier chunks, earlier threads of the chunk and earlier items of the
// thread, so every pass is stable.  The passes alternate between the
// bucket's entries (overwritten: they are scratch once read) and the output;
// the result ends in the output.  Cost: (bits / 4) passes of two reads and
// one write per entry, on one SM; buckets this large come only from
// degenerate inputs (piles) or mass deletion.
#pragma once
#include <cstdint>

namespace pbf103 {

constexpr uint32_t kRadixThreads = 256;
constexpr uint32_t kRadixItems = 8;
constexpr uint32_t kRadixChunk = kRadixThreads * kRadixItems;

// shared memory of the sort: per digit and thread, counts and then their
// exclusive prefixes over the chunk's threads (16 KB)
struct RadixSmem {
    uint32_t cnt[16][kRadixThreads];
};

// index bits of indices below `bound`
__host__ __device__ __forceinline__ uint32_t radix_bits(uint32_t bound)
{
    uint32_t b = 1;
    while (b < 32 && (bound - 1u) >> b) ++b;
    return b;
}

// Sorts the b entries of `a` by (entry & imask) into `out` (masked values).
// `a` is overwritten.  Every thread of the block must call it with the same
// arguments; blockDim.x == kRadixThreads.
__device__ inline void block_radix_stable(uint32_t *a, uint32_t *out, uint32_t b, uint32_t imask, uint32_t nbits,
                                   RadixSmem &sm, uint32_t *base /* __shared__ [16] */,
                                   uint32_t *tot /* __shared__ [16] */)
{
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint32_t passes = (nbits + 3u) / 4u;
    // passes alternate a -> out -> a ...; an even count ends in a, so the
    // first pass then writes back into a (stable in place is not possible):
    // start from out instead, after copying the masked entries there
    uint32_t *src = a, *dst = out;
    if ((passes & 1u) == 0u) {
        for (uint32_t i = t; i < b; i += kRadixThreads) out[i] = a[i] & imask;
        __syncthreads();
        src = out;
        dst = a;
    }
    for (uint32_t p = 0; p < passes; ++p) {
        const uint32_t shift = 4u * p;
        const uint32_t m = (p == 0 && src == a) ? imask : 0xFFFFFFFFu;
        if (t < 16) base[t] = 0;
        __syncthreads();
        for (uint32_t i = t; i < b; i += kRadixThreads) atomicAdd(&base[((src[i] & m) >> shift) & 15u], 1u);
        __syncthreads();
        if (t == 0) {
            uint32_t run = 0;
            for (uint32_t d = 0; d < 16; ++d) {
                const uint32_t c = base[d];
                base[d] = run;
                run += c;
            }
        }
        __syncthreads();
        for (uint32_t c0 = 0; c0 < b; c0 += kRadixChunk) {
            uint32_t v[kRadixItems];
            uint64_t packed = 0;  // 16 digits x 4-bit counts of this thread's items (at most 8 each)
#pragma unroll
            for (uint32_t k = 0; k < kRadixItems; ++k) {
                const uint32_t idx = c0 + kRadixItems * t + k;
                v[k] = idx < b ? (src[idx] & m) : 0u;
                if (idx < b) packed += 1ull << (4u * (((v[k] >> shift) & 15u)));
            }
#pragma unroll
            for (uint32_t d = 0; d < 16; ++d) sm.cnt[d][t] = (uint32_t)(packed >> (4u * d)) & 15u;
            __syncthreads();
            // exclusive prefix over the chunk's threads, two digits per warp:
            // lane L takes threads 8L .. 8L+7
#pragma unroll
            for (uint32_t dd = 0; dd < 2; ++dd) {
                const uint32_t d = 2u * warp + dd;
                uint32_t loc[8], s = 0;
#pragma unroll
                for (uint32_t j = 0; j < 8; ++j) {
                    loc[j] = s;
                    s += sm.cnt[d][8u * lane + j];
                }
                uint32_t inc = s;
#pragma unroll
                for (uint32_t o = 1; o < 32; o <<= 1) {
                    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += u;
                }
                const uint32_t pre = inc - s;
#pragma unroll
                for (uint32_t j = 0; j < 8; ++j) sm.cnt[d][8u * lane + j] = pre + loc[j];
                if (lane == 31) tot[d] = inc;
            }
            __syncthreads();
            uint64_t seen = 0;
#pragma unroll
            for (uint32_t k = 0; k < kRadixItems; ++k) {
                const uint32_t idx = c0 + kRadixItems * t + k;
                if (idx < b) {
                    const uint32_t d = (v[k] >> shift) & 15u;
                    const uint32_t off = (uint32_t)(seen >> (4u * d)) & 15u;
                    seen += 1ull << (4u * d);
                    dst[base[d] + sm.cnt[d][t] + off] = v[k];
                }
            }
            __syncthreads();
            if (t < 16) base[t] += tot[t];
            __syncthreads();
        }
        uint32_t *tmp = src;
        src = dst;
        dst = tmp;
        __syncthreads();
    }
}

}  // namespace pbf103
