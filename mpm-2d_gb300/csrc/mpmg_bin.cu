// Element binning of the step: a counting sort of (element key, storage
// position) pairs that gives the same order as a stable sort by key (hence
// the reference's per-element order, process_usl.c:677-723).
//
//   count    bins[key] for keys inside the grid (warp-aggregated atomics),
//            bins[ne + b] = keys outside the grid in 256-key block b.  The
//            kernel that produces the keys does this (mpmg_bin_count_block);
//            mpmg_bin_count launches it stand-alone when it did not.
//   scan     exclusive prefix of all bins (reduce-then-scan, three small
//            kernels): element starts (cell_start) and scatter cursors; the
//            bins go back to zero for the next step.
//   scatter  every key takes a slot of its element (warp-aggregated
//            atomics); keys outside the grid go straight to their final
//            place in storage order (block start + rank in the block).
//   order    each element's few slots are sorted by storage position where
//            they are consumed (the P2G kernels, mpmg_order_segment), which
//            makes the whole permutation stable and deterministic whatever
//            order the atomics ran in.
#include "mpmg_internal.cuh"

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(256) count_kernel(const uint32_t *__restrict__ keys, int n, uint32_t sentinel,
                                                    uint32_t *__restrict__ bins)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    mpmg_bin_count_block(k < n ? keys[k] : 0xffffffffu, k < n, sentinel, bins);
}

// Sum of each tile of bins.
__global__ void __launch_bounds__(kScanThreads) tile_sum_kernel(const uint32_t *__restrict__ bins, int m,
                                                                uint32_t *__restrict__ tile_sums)
{
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const int base = blockIdx.x * kScanTile;
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        int idx = base + j * kScanThreads + threadIdx.x;
        if (idx < m) s += bins[idx];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += warp_sums[w];
        tile_sums[blockIdx.x] = t;
    }
}

// Exclusive scan of the tile sums in place (one block; loops over chunks).
__global__ void __launch_bounds__(1024) tile_scan_kernel(uint32_t *__restrict__ tile_sums, int tiles)
{
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < tiles; base += 1024) {
        const int idx = base + threadIdx.x;
        const uint32_t v = idx < tiles ? tile_sums[idx] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += u;
        }
        if (lane == 31) warp_tot[w] = incl;
        __syncthreads();
        uint32_t wbase = 0;
        for (int j = 0; j < w; j++) wbase += warp_tot[j];
        const uint32_t c = carry;
        if (idx < tiles) tile_sums[idx] = c + wbase + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + wbase + incl;
        __syncthreads();
    }
}

// Exclusive scan of each tile of bins plus its tile offset: cursors for all
// bins, cell_start for elements 0..ne (ne: the first outside bin, i.e. the
// number of particles inside); the bins go back to zero.
__global__ void __launch_bounds__(kScanThreads) tile_scan_write_kernel(uint32_t *__restrict__ bins, int m, int ne,
                                                                       const uint32_t *__restrict__ tile_offsets,
                                                                       int *__restrict__ cell_start,
                                                                       uint32_t *__restrict__ cursor)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;   // 8 consecutive bins per thread
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        int idx = base + j;
        v[j] = idx < m ? bins[idx] : 0u;
        s += v[j];
    }
    uint32_t incl = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += u;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    uint32_t run = tile_offsets[blockIdx.x] + incl - s;
    for (int j = 0; j < w; j++) run += warp_tot[j];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        int idx = base + j;
        if (idx < m) {
            if (idx <= ne) cell_start[idx] = (int)run;
            cursor[idx] = run;
            bins[idx] = 0;
        }
        run += v[j];
    }
}

__global__ void __launch_bounds__(256) scatter_kernel(const uint32_t *__restrict__ keys, int n, uint32_t sentinel,
                                                      uint32_t *__restrict__ cursor, uint32_t *__restrict__ slots,
                                                      uint32_t *__restrict__ perm,
                                                      uint32_t *__restrict__ sorted_keys)
{
    __shared__ uint32_t warp_out[8];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const bool valid = k < n;
    const uint32_t key = valid ? keys[k] : 0xffffffffu;
    const bool out = valid && key == sentinel;
    const uint32_t outside = __ballot_sync(0xffffffffu, out);
    const uint32_t vmask = __ballot_sync(0xffffffffu, valid && !out);   // before any lane leaves
    if (lane == 0) warp_out[w] = __popc(outside);
    __syncthreads();
    if (out) {
        uint32_t r = __popc(outside & lt);
        for (int j = 0; j < w; j++) r += warp_out[j];
        const uint32_t pos = cursor[sentinel + blockIdx.x] + r;
        perm[pos] = (uint32_t)k;          // final: storage order within the block's run
        sorted_keys[pos] = key;
        return;
    }
    if (!valid) return;
    const uint32_t peers = __match_any_sync(vmask, key);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&cursor[key], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const uint32_t pos = base + __popc(peers & lt);
    slots[pos] = (uint32_t)k;
    sorted_keys[pos] = key;
}

}  // namespace

int mpmg_bin_init(mpmg_ctx *ctx)
{
    const size_t blocks = (ctx->np + 255) / 256;
    const size_t m = ctx->ne + (blocks ? blocks : 1);
    const size_t tiles = (m + kScanTile - 1) / kScanTile;
    MPMG_CHECK(cudaMalloc(&ctx->bin.counts, m * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->bin.cursor, m * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->bin.tile_sums, (tiles ? tiles : 1) * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->bin.slots, (ctx->np ? ctx->np : 1) * sizeof(uint32_t)));
    MPMG_CHECK(cudaMemsetAsync(ctx->bin.counts, 0, m * sizeof(uint32_t), ctx->stream));
    ctx->bin.bins = (int)m;
    ctx->bin.tiles = (int)tiles;
    return MPMG_OK;
}

void mpmg_bin_free(mpmg_ctx *ctx)
{
    cudaFree(ctx->bin.counts);
    cudaFree(ctx->bin.cursor);
    cudaFree(ctx->bin.tile_sums);
    cudaFree(ctx->bin.slots);
    ctx->bin.counts = ctx->bin.cursor = ctx->bin.tile_sums = ctx->bin.slots = nullptr;
}

int mpmg_bin_count(mpmg_ctx *ctx, const uint32_t *keys)
{
    const int n = (int)ctx->np;
    if (n > 0) {
        count_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(keys, n, (uint32_t)ctx->ne, ctx->bin.counts);
        ctx->launches += 1;
    }
    return MPMG_OK;
}

// Scan of the counted bins and scatter of keys[n]: cell_start[ne + 1],
// sorted_keys[n], perm[k] for keys outside the grid and bin.slots (unordered
// within each element) for the rest.
int mpmg_bin_scan_scatter(mpmg_ctx *ctx, const uint32_t *keys)
{
    cudaStream_t s = ctx->stream;
    const int n = (int)ctx->np;
    const int m = ctx->bin.bins;
    const int tiles = ctx->bin.tiles;
    tile_sum_kernel<<<tiles, kScanThreads, 0, s>>>(ctx->bin.counts, m, ctx->bin.tile_sums);
    tile_scan_kernel<<<1, 1024, 0, s>>>(ctx->bin.tile_sums, tiles);
    tile_scan_write_kernel<<<tiles, kScanThreads, 0, s>>>(ctx->bin.counts, m, (int)ctx->ne, ctx->bin.tile_sums,
                                                          ctx->cell_start, ctx->bin.cursor);
    ctx->launches += 3;
    if (n > 0) {
        scatter_kernel<<<(n + 255) / 256, 256, 0, s>>>(keys, n, (uint32_t)ctx->ne, ctx->bin.cursor, ctx->bin.slots,
                                                       ctx->perm, ctx->sorted_keys);
        ctx->launches += 1;
    }
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}
