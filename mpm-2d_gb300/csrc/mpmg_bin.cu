// Element binning of the step: a counting sort of (element key, storage
// position) pairs that gives the same order as a stable sort by key (hence
// the reference's per-element order, process_usl.c:677-723).
//
//   count    bins[key] for keys inside the grid (warp-aggregated atomics),
//            bins[ne + g] = keys outside the grid at storage positions
//            32 g .. 32 g + 31.  The kernel that produces the keys does this
//            (mpmg_bin_count); the count kernel here runs it stand-alone.
//   scan     exclusive prefix of all bins in one pass (decoupled
//            look-back): element starts (cell_start) and scatter cursors; the
//            bins go back to zero for the next step.
//   scatter  every key takes a slot of its element (warp-aggregated
//            atomics); keys outside the grid go straight to their final
//            place in storage order (group start + rank in the group).
//   order    each element's few slots are sorted by storage position where
//            they are consumed (the P2G kernels, mpmg_order_segment), which
//            makes the whole permutation stable and deterministic whatever
//            order the atomics ran in; the same pass writes the inverse
//            permutation (rank).
#include "mpmg_internal.cuh"

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(256) count_kernel(const uint32_t *__restrict__ keys, int n, uint32_t sentinel,
                                                    uint32_t *__restrict__ bins)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    mpmg_bin_count(k < n ? keys[k] : 0u, k < n, sentinel, (uint32_t)k >> 5, bins);
}

// Single-pass exclusive scan of the bins (decoupled look-back): each block
// takes the next tile by ticket, publishes its tile total, then walks back
// over earlier tiles' published totals (or inclusive prefixes) to find its
// offset, publishes its inclusive prefix, and writes cursors, cell_start and
// zeroed bins.  Tiles are taken in ticket order, so every tile a block waits
// for belongs to a block that started earlier; each wait is still bounded,
// and on a timeout the kernel sets MPMG_DEV_ERR_SPIN and stops.
constexpr uint64_t kFlagAggregate = 1ull << 62;
constexpr uint64_t kFlagInclusive = 2ull << 62;
constexpr uint64_t kValueMask = (1ull << 62) - 1;
constexpr long long kLookbackSpinLimit = 1 << 24;

__global__ void __launch_bounds__(kScanThreads) scan_kernel(uint32_t *__restrict__ bins, int m, int ne,
                                                            unsigned long long *__restrict__ tile_state,
                                                            unsigned int *__restrict__ ticket,
                                                            int *__restrict__ cell_start,
                                                            uint32_t *__restrict__ cursor, int *status)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    __shared__ int tile_s;
    __shared__ uint32_t prefix_s;
    __shared__ int abort_s;
    if (threadIdx.x == 0) {
        tile_s = (int)atomicAdd(ticket, 1u);
        abort_s = 0;
    }
    __syncthreads();
    const int tile = tile_s;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int base = tile * kScanTile + threadIdx.x * kScanItems;   // 8 consecutive bins per thread
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const int idx = base + j;
        v[j] = idx < m ? bins[idx] : 0u;
        sum += v[j];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += u;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (int j = 0; j < kScanThreads / 32; j++) total += warp_tot[j];
        volatile unsigned long long *st = tile_state;
        if (tile == 0) {
            st[0] = kFlagInclusive | total;
            prefix_s = 0;
        } else {
            st[tile] = kFlagAggregate | total;
            __threadfence();
            uint32_t prefix = 0;
            int p = tile - 1;
            long long spins = 0;
            while (p >= 0) {
                const unsigned long long word = st[p];
                if ((word & ~kValueMask) == 0) {
                    if (++spins > kLookbackSpinLimit) {
                        atomicOr(status, MPMG_DEV_ERR_SPIN);
                        abort_s = 1;
                        break;
                    }
                    continue;
                }
                prefix += (uint32_t)(word & kValueMask);
                if (word & kFlagInclusive) break;
                p--;
            }
            __threadfence();
            st[tile] = kFlagInclusive | (unsigned long long)(prefix + total);
            prefix_s = prefix;
        }
    }
    __syncthreads();
    if (abort_s) return;
    uint32_t run = prefix_s + incl - sum;
    for (int j = 0; j < w; j++) run += warp_tot[j];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        const int idx = base + j;
        if (idx < m) {
            if (idx <= ne) cell_start[idx] = (int)run;
            cursor[idx] = run;
            bins[idx] = 0;
        }
        run += v[j];
    }
}

// Each warp scatters 4 consecutive groups of 32 keys (independent
// iterations: several atomics and stores in flight per lane).
constexpr int kScatterGroups = 4;

__global__ void __launch_bounds__(256) scatter_kernel(const uint32_t *__restrict__ keys, int n, uint32_t sentinel,
                                                      uint32_t *__restrict__ cursor, uint32_t *__restrict__ slots,
                                                      uint32_t *__restrict__ perm, uint32_t *__restrict__ rank,
                                                      uint32_t *__restrict__ sorted_keys)
{
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
#pragma unroll
    for (int j = 0; j < kScatterGroups; j++) {
        const int group = warp_global * kScatterGroups + j;
        const int k = group * 32 + lane;
        const bool valid = k < n;
        const uint32_t key = valid ? keys[k] : 0u;
        const bool out = valid && key == sentinel;
        const bool in = valid && key != sentinel;
        const uint32_t outside = __ballot_sync(0xffffffffu, out);
        const uint32_t inmask = __ballot_sync(0xffffffffu, in);
        if (out) {
            const uint32_t pos = cursor[sentinel + group] + __popc(outside & lt);
            perm[pos] = (uint32_t)k;      // final: storage order within the group's run
            rank[k] = pos;
            sorted_keys[pos] = key;
        }
        if (in) {
            const uint32_t peers = __match_any_sync(inmask, key);
            const int leader = __ffs(peers) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&cursor[key], (uint32_t)__popc(peers));
            base = __shfl_sync(peers, base, leader);
            const uint32_t pos = base + __popc(peers & lt);
            slots[pos] = (uint32_t)k;
            sorted_keys[pos] = key;
        }
    }
}

}  // namespace

int mpmg_bin_init(mpmg_ctx *ctx)
{
    const size_t groups = (ctx->np + 31) / 32;
    const size_t m = ctx->ne + (groups ? groups : 1);
    const size_t tiles = (m + kScanTile - 1) / kScanTile;
    MPMG_CHECK(cudaMalloc(&ctx->bin.counts, m * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->bin.cursor, m * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->bin.tile_state, (tiles ? tiles : 1) * sizeof(unsigned long long) + 16));
    MPMG_CHECK(cudaMalloc(&ctx->bin.slots, (ctx->np ? ctx->np : 1) * sizeof(uint32_t)));
    MPMG_CHECK(cudaMalloc(&ctx->bin.rank, (ctx->np ? ctx->np : 1) * sizeof(uint32_t)));
    MPMG_CHECK(cudaMemsetAsync(ctx->bin.counts, 0, m * sizeof(uint32_t), ctx->stream));
    ctx->bin.bins = (int)m;
    ctx->bin.tiles = (int)tiles;
    return MPMG_OK;
}

void mpmg_bin_free(mpmg_ctx *ctx)
{
    cudaFree(ctx->bin.counts);
    cudaFree(ctx->bin.cursor);
    cudaFree(ctx->bin.tile_state);
    cudaFree(ctx->bin.slots);
    cudaFree(ctx->bin.rank);
    ctx->bin.counts = ctx->bin.cursor = ctx->bin.slots = ctx->bin.rank = nullptr;
    ctx->bin.tile_state = nullptr;
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
// sorted_keys[n], perm and rank for keys outside the grid, and bin.slots
// (unordered within each element) for the rest.
int mpmg_bin_scan_scatter(mpmg_ctx *ctx, const uint32_t *keys)
{
    cudaStream_t s = ctx->stream;
    const int n = (int)ctx->np;
    const int m = ctx->bin.bins;
    const int tiles = ctx->bin.tiles;
    // tile states and the ticket counter (right after them) start at zero
    MPMG_CHECK(cudaMemsetAsync(ctx->bin.tile_state, 0, (size_t)tiles * sizeof(unsigned long long) + 16, s));
    unsigned int *ticket = (unsigned int *)(ctx->bin.tile_state + tiles);
    scan_kernel<<<tiles, kScanThreads, 0, s>>>(ctx->bin.counts, m, (int)ctx->ne, ctx->bin.tile_state, ticket,
                                               ctx->cell_start, ctx->bin.cursor, ctx->d_status);
    ctx->launches += 1;
    if (n > 0) {
        const int keys_per_block = 256 * kScatterGroups;
        scatter_kernel<<<(n + keys_per_block - 1) / keys_per_block, 256, 0, s>>>(
            keys, n, (uint32_t)ctx->ne, ctx->bin.cursor, ctx->bin.slots, ctx->perm, ctx->bin.rank, ctx->sorted_keys);
        ctx->launches += 1;
    }
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}
