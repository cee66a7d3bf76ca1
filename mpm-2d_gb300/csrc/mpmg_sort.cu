// Stable LSD radix sort of (element key, particle index) pairs, and the
// per-element start offsets of the sorted order.
//
// The reference groups particles by element in find_filled_elements
// (libmpm/process_usl.c:677-723): for each element, its particles in
// ascending particle index.  A stable sort of the keys over particle indices
// 0..n-1 reproduces exactly those groups, so the permutation is bit-exact
// against the reference's lists.
//
// Each pass sorts one 8-bit digit in three launches:
//   upsweep    per-tile digit histogram (tile = 2048 keys)
//   scan       exclusive scan of the digit-major [256][tiles] histogram
//   downsweep  stable in-tile rank (warp match + per-warp counts) and scatter
// Integer-only, no floating point, deterministic for any launch order.
#include "mpmg_internal.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;
constexpr int kRadix = 256;
constexpr int kWarps = kThreads / 32;

__global__ void __launch_bounds__(kThreads) upsweep_kernel(const uint32_t *__restrict__ keys, int n,
                                                           int shift, int num_tiles,
                                                           uint32_t *__restrict__ tile_hist)
{
    __shared__ uint32_t hist[kRadix];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kTile;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        int idx = base + k * kThreads + threadIdx.x;
        if (idx < n) {
            uint32_t d = (keys[idx] >> shift) & (kRadix - 1);
            atomicAdd(&hist[d], 1u);
        }
    }
    __syncthreads();
    tile_hist[threadIdx.x * num_tiles + blockIdx.x] = hist[threadIdx.x];
}

// Exclusive scan of len entries by one block of 1024 threads.
__global__ void __launch_bounds__(1024) scan_kernel(uint32_t *__restrict__ data, int len)
{
    __shared__ uint32_t sums[1024];
    const int per = (len + 1023) / 1024;
    const int begin = threadIdx.x * per;
    const int end = min(begin + per, len);
    uint32_t local = 0;
    for (int i = begin; i < end; i++) local += data[i];
    sums[threadIdx.x] = local;
    __syncthreads();
    // Hillis-Steele inclusive scan over the 1024 partial sums.
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = (threadIdx.x >= off) ? sums[threadIdx.x - off] : 0u;
        __syncthreads();
        sums[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = (threadIdx.x == 0) ? 0u : sums[threadIdx.x - 1];
    for (int i = begin; i < end; i++) {
        uint32_t v = data[i];
        data[i] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kThreads) downsweep_kernel(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in, int n, int shift,
    int num_tiles, const uint32_t *__restrict__ tile_offsets, uint32_t *__restrict__ keys_out,
    uint32_t *__restrict__ vals_out)
{
    __shared__ uint32_t offsets[kRadix];
    __shared__ uint32_t warp_counts[kWarps][kRadix];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    offsets[threadIdx.x] = tile_offsets[threadIdx.x * num_tiles + blockIdx.x];
    const int base = blockIdx.x * kTile;

    for (int k = 0; k < kItems; k++) {
#pragma unroll
        for (int w = 0; w < kWarps; w++) warp_counts[w][threadIdx.x] = 0;
        __syncthreads();
        const int idx = base + k * kThreads + threadIdx.x;
        const bool valid = idx < n;
        uint32_t key = 0, val = 0, d = 0;
        if (valid) {
            key = keys_in[idx];
            val = vals_in[idx];
            d = (key >> shift) & (kRadix - 1);
        }
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 0xffffffffu) & vmask;
        uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) warp_counts[warp][d] = __popc(peers);
        __syncthreads();
        // Digit threadIdx.x: exclusive prefix over warps, then advance the tile offset.
        {
            uint32_t run = offsets[threadIdx.x];
#pragma unroll
            for (int w = 0; w < kWarps; w++) {
                uint32_t c = warp_counts[w][threadIdx.x];
                warp_counts[w][threadIdx.x] = run;
                run += c;
            }
            offsets[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t dst = warp_counts[warp][d] + rank;
            keys_out[dst] = key;
            vals_out[dst] = val;
        }
        __syncthreads();
    }
}

// cell_start[e] = first sorted position whose key is >= e, for e in [0, ne].
__global__ void cell_start_kernel(const uint32_t *__restrict__ sorted_keys, int n, int ne,
                                  int *__restrict__ cell_start)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e > ne) return;
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (sorted_keys[mid] < (uint32_t)e) lo = mid + 1;
        else hi = mid;
    }
    cell_start[e] = lo;
}

}  // namespace

int mpmg_sort_init(mpmg_ctx *ctx)
{
    int n = (int)ctx->np;
    ctx->sort.capacity = n;
    ctx->sort.num_tiles = (n + kTile - 1) / kTile;
    if (ctx->sort.num_tiles < 1) ctx->sort.num_tiles = 1;
    size_t cap = (size_t)(n > 0 ? n : 1);
    MPMG_CHECK(cudaMalloc(&ctx->sort.keys_alt, cap * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->sort.vals_alt, cap * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->sort.tile_hist, (size_t)kRadix * ctx->sort.num_tiles * sizeof(uint32_t)));
    return MPMG_OK;
}

void mpmg_sort_free(mpmg_ctx *ctx)
{
    cudaFree(ctx->sort.keys_alt);
    cudaFree(ctx->sort.vals_alt);
    cudaFree(ctx->sort.tile_hist);
    ctx->sort.keys_alt = ctx->sort.vals_alt = ctx->sort.tile_hist = nullptr;
}

// Sorts (ctx->keys, ctx->vals) into (ctx->sorted_keys, ctx->perm) and fills
// ctx->cell_start.
int mpmg_sort_keys(mpmg_ctx *ctx)
{
    const int n = (int)ctx->np;
    const int ne = (int)ctx->ne;
    const int passes = (ctx->key_bits + 7) / 8;
    const int tiles = ctx->sort.num_tiles;
    cudaStream_t s = ctx->stream;
    if (n > 0) {
        const uint32_t *src_k = ctx->keys, *src_v = ctx->vals;
        for (int p = 0; p < passes; p++) {
            bool to_out = ((passes - 1 - p) % 2) == 0;
            uint32_t *dst_k = to_out ? ctx->sorted_keys : ctx->sort.keys_alt;
            uint32_t *dst_v = to_out ? ctx->perm : ctx->sort.vals_alt;
            int shift = 8 * p;
            upsweep_kernel<<<tiles, kThreads, 0, s>>>(src_k, n, shift, tiles, ctx->sort.tile_hist);
            scan_kernel<<<1, 1024, 0, s>>>(ctx->sort.tile_hist, kRadix * tiles);
            downsweep_kernel<<<tiles, kThreads, 0, s>>>(src_k, src_v, n, shift, tiles, ctx->sort.tile_hist,
                                                        dst_k, dst_v);
            ctx->launches += 3;
            src_k = dst_k;
            src_v = dst_v;
        }
    }
    cell_start_kernel<<<(ne + 1 + 255) / 256, 256, 0, s>>>(ctx->sorted_keys, n, ne, ctx->cell_start);
    ctx->launches += 1;
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}
