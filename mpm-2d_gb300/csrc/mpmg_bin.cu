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
//            bins go back to zero for the next step, and nothing else needs
//            clearing between steps.
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
constexpr int kScanItems = 8;      // 2048 bins a tile, spread over many SMs: measured fastest on the step
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(256) count_kernel(const uint32_t *__restrict__ keys, int n, uint32_t sentinel,
                                                    uint32_t *__restrict__ bins)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    mpmg_bin_count(k < n ? keys[k] : 0u, k < n, sentinel, (uint32_t)k >> 5, bins);
}

// Single-pass exclusive scan of the bins (decoupled look-back).  Each block
// takes the next tile by ticket (atomicInc wraps the ticket back to 0 after
// the last tile, so it never needs resetting), publishes its tile total, and
// warp 0 looks back over the previous 32 tiles at a time: it folds in
// published totals until it reaches an inclusive prefix.  Tiles are taken in
// ticket order, so every tile a block waits for belongs to a block that
// started earlier; each wait is still bounded, and on a timeout the kernel
// sets MPMG_DEV_ERR_SPIN and stops.
//
// A tile state word is  flag (2 bits) | epoch (30 bits) | value (32 bits).
// The epoch is a launch counter kept after the ticket: states written by an
// earlier launch carry an older epoch and read as "not yet published", so
// the states need no clearing between launches.  The block that takes the
// last tile advances the epoch once its own look-back is complete, which
// happens only after every tile of the launch has published (and so has
// read the epoch).
constexpr uint64_t kFlagAggregate = 1ull << 62;
constexpr uint64_t kFlagInclusive = 2ull << 62;
constexpr uint64_t kFlagMask = 3ull << 62;
constexpr uint32_t kEpochMask = (1u << 30) - 1u;
constexpr long long kLookbackSpinLimit = 1 << 22;

__device__ __forceinline__ uint32_t warp_sum(uint32_t v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__global__ void __launch_bounds__(kScanThreads) scan_kernel(uint32_t *__restrict__ bins, int m, int ne,
                                                            unsigned long long *__restrict__ tile_state,
                                                            unsigned int *__restrict__ ticket_epoch,
                                                            int *__restrict__ cell_start,
                                                            uint32_t *__restrict__ cursor, int *status)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    __shared__ int tile_s;
    __shared__ uint32_t epoch_s;
    __shared__ uint32_t prefix_s;
    __shared__ int abort_s;
    if (threadIdx.x == 0) {
        // ticket and epoch belong to the scan alone (the previous scan has
        // completed): taken before waiting for the kernel that counted the bins
        tile_s = (int)atomicInc(&ticket_epoch[0], gridDim.x - 1u);
        epoch_s = *(volatile unsigned int *)&ticket_epoch[1] & kEpochMask;
        abort_s = 0;
    }
    mpmg_pdl_wait();
    mpmg_pdl_trigger();
    __syncthreads();
    const int tile = tile_s;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int base = tile * kScanTile + threadIdx.x * kScanItems;   // kScanItems consecutive bins per thread
    uint32_t v[kScanItems];
    uint32_t sum = 0;
    if (base + kScanItems <= m) {
#pragma unroll
        for (int j = 0; j < kScanItems; j += 4) {
            const uint4 q = *reinterpret_cast<const uint4 *>(bins + base + j);
            v[j] = q.x;
            v[j + 1] = q.y;
            v[j + 2] = q.z;
            v[j + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < kScanItems; j++) v[j] = base + j < m ? bins[base + j] : 0u;
    }
#pragma unroll
    for (int j = 0; j < kScanItems; j++) sum += v[j];
    uint32_t incl = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += u;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        const uint32_t epoch = epoch_s;
        const uint64_t tag = (uint64_t)epoch << 32;
        const uint32_t total = warp_sum(lane < kScanThreads / 32 ? warp_tot[lane] : 0u);
        volatile unsigned long long *st = tile_state;
        uint32_t prefix = 0;
        bool ok = true;
        if (tile == 0) {
            if (lane == 0) st[0] = kFlagInclusive | tag | total;
        } else {
            if (lane == 0) st[tile] = kFlagAggregate | tag | total;
            int p = tile - 1;      // newest tile not yet folded in
            long long polls = 0;
            while (true) {
                const int q = p - lane;
                const uint64_t word = q >= 0 ? st[q] : (kFlagInclusive | tag);   // before tile 0: zero
                const bool ready = (word & kFlagMask) != 0 && (uint32_t)((word >> 32) & kEpochMask) == epoch;
                const uint32_t incl_mask = __ballot_sync(0xffffffffu, ready && (word & kFlagInclusive) != 0);
                const int last = incl_mask ? __ffs(incl_mask) - 1 : 31;   // lanes 0..last are needed
                const uint32_t need = (2u << last) - 1u;
                const uint32_t ready_mask = __ballot_sync(0xffffffffu, ready);
                if ((ready_mask & need) != need) {
                    if (++polls > kLookbackSpinLimit) {
                        ok = false;
                        break;
                    }
                    continue;
                }
                prefix += warp_sum(lane <= last ? (uint32_t)word : 0u);
                if (incl_mask) break;
                p -= 32;
            }
            // flag and value travel in one word, and the value depends on
            // every state folded in, so no fence is needed before it
            if (ok && lane == 0) st[tile] = kFlagInclusive | tag | (uint64_t)(uint32_t)(prefix + total);
        }
        if (lane == 0) {
            prefix_s = prefix;
            if (!ok) {
                atomicOr(status, MPMG_DEV_ERR_SPIN);
                abort_s = 1;
            } else if (tile == (int)gridDim.x - 1) {
                // every tile has published: the next launch may start a new epoch
                __threadfence();
                *(volatile unsigned int *)&ticket_epoch[1] = (epoch + 1u) & kEpochMask;
            }
        }
    }
    __syncthreads();
    if (abort_s) return;
    uint32_t run = prefix_s + incl - sum;
    for (int j = 0; j < w; j++) run += warp_tot[j];
    uint32_t ex[kScanItems];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        ex[j] = run;
        run += v[j];
    }
    if (base + kScanItems <= m) {
#pragma unroll
        for (int j = 0; j < kScanItems; j += 4) {
            *reinterpret_cast<uint4 *>(cursor + base + j) = make_uint4(ex[j], ex[j + 1], ex[j + 2], ex[j + 3]);
            *reinterpret_cast<uint4 *>(bins + base + j) = make_uint4(0u, 0u, 0u, 0u);
        }
    } else {
#pragma unroll
        for (int j = 0; j < kScanItems; j++)
            if (base + j < m) {
                cursor[base + j] = ex[j];
                bins[base + j] = 0u;
            }
    }
    if (base + kScanItems <= ne + 1) {
#pragma unroll
        for (int j = 0; j < kScanItems; j += 4)
            *reinterpret_cast<int4 *>(cell_start + base + j) =
                make_int4((int)ex[j], (int)ex[j + 1], (int)ex[j + 2], (int)ex[j + 3]);
    } else if (base <= ne) {
#pragma unroll
        for (int j = 0; j < kScanItems; j++)
            if (base + j <= ne) cell_start[base + j] = (int)ex[j];
    }
}

// Each warp scatters 4 consecutive groups of 32 keys.  Within a group, each
// run of equal keys in consecutive lanes takes its slots with one atomic
// (the keys arrive nearly sorted, so a group holds a few runs); the groups'
// atomics are all issued before any result is used, so a lane has its four
// atomics in flight at once.
constexpr int kScatterGroups = 4;

__global__ void __launch_bounds__(256) scatter_kernel(const uint32_t *__restrict__ keys, int n, uint32_t sentinel,
                                                      uint32_t *__restrict__ cursor, uint32_t *__restrict__ slots,
                                                      uint32_t *__restrict__ perm, uint32_t *__restrict__ rank,
                                                      uint32_t *__restrict__ sorted_keys)
{
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t key[kScatterGroups], starts[kScatterGroups], base[kScatterGroups], outside[kScatterGroups];
#pragma unroll
    for (int j = 0; j < kScatterGroups; j++) {
        const int k = (warp_global * kScatterGroups + j) * 32 + lane;
        key[j] = k < n ? keys[k] : sentinel + 1u;     // sentinel + 1: no key
    }
    // the keys come from before the scan; the cursors from the scan
    mpmg_pdl_wait();
#pragma unroll
    for (int j = 0; j < kScatterGroups; j++) {
        const bool in = key[j] < sentinel;
        const uint32_t b = in ? key[j] : 0xffffffffu;
        const uint32_t prev = __shfl_up_sync(0xffffffffu, b, 1);
        const bool start = in && (lane == 0 || prev != b);
        starts[j] = __ballot_sync(0xffffffffu, start);
        outside[j] = __ballot_sync(0xffffffffu, key[j] == sentinel);
        const uint32_t invalid = ~__ballot_sync(0xffffffffu, in);
        base[j] = 0;
        if (start) {
            const uint32_t above = lane == 31 ? 0u : (starts[j] | invalid) & (0xfffffffeu << lane);
            const int end = above ? __ffs(above) - 1 : 32;
            base[j] = atomicAdd(&cursor[key[j]], (uint32_t)(end - lane));
        }
    }
    mpmg_pdl_trigger();
#pragma unroll
    for (int j = 0; j < kScatterGroups; j++) {
        const int group = warp_global * kScatterGroups + j;
        const int k = group * 32 + lane;
        const uint32_t below = starts[j] & (lt | (1u << lane));
        const int leader = below ? 31 - __clz(below) : lane;
        const uint32_t b = __shfl_sync(0xffffffffu, base[j], leader);
        if (key[j] == sentinel) {
            const uint32_t pos = cursor[sentinel + group] + __popc(outside[j] & lt);
            perm[pos] = (uint32_t)k;      // final: storage order within the group's run
            rank[k] = pos;
            if (sorted_keys != nullptr) sorted_keys[pos] = key[j];
        } else if (key[j] < sentinel) {
            const uint32_t pos = b + (uint32_t)(lane - leader);
            slots[pos] = (uint32_t)k;
            if (sorted_keys != nullptr) sorted_keys[pos] = key[j];
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
    // tile states, ticket and epoch start at zero (no tile published)
    MPMG_CHECK(cudaMemsetAsync(ctx->bin.tile_state, 0, (tiles ? tiles : 1) * sizeof(unsigned long long) + 16,
                               ctx->stream));
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

// Back to the initial look-back state, after a launch that stopped on a
// timed-out wait left some tiles of its epoch unpublished.
int mpmg_bin_reset(mpmg_ctx *ctx)
{
    if (ctx->bin.tile_state == nullptr) return MPMG_OK;
    MPMG_CHECK(cudaMemset(ctx->bin.tile_state, 0,
                          (size_t)(ctx->bin.tiles ? ctx->bin.tiles : 1) * sizeof(unsigned long long) + 16));
    MPMG_CHECK(cudaMemset(ctx->bin.counts, 0, (size_t)ctx->bin.bins * sizeof(uint32_t)));
    return MPMG_OK;
}

// Scan of the counted bins and scatter of keys[n]: cell_start[ne + 1],
// perm and rank for keys outside the grid, bin.slots (unordered within each
// element) for the rest, and sorted_keys[n] unless it is null.
int mpmg_bin_scan_scatter(mpmg_ctx *ctx, const uint32_t *keys, uint32_t *sorted_keys, bool pdl)
{
    cudaStream_t s = ctx->stream;
    const int n = (int)ctx->np;
    const int m = ctx->bin.bins;
    const int tiles = ctx->bin.tiles;
    unsigned int *ticket_epoch = (unsigned int *)(ctx->bin.tile_state + tiles);
    MPMG_CHECK(mpmg_launch_pdl(pdl, scan_kernel, dim3(tiles), dim3(kScanThreads), 0, s, ctx->bin.counts, m,
                               (int)ctx->ne, ctx->bin.tile_state, ticket_epoch, ctx->cell_start, ctx->bin.cursor,
                               ctx->d_status));
    ctx->launches += 1;
    if (n > 0) {
        const int keys_per_block = 256 * kScatterGroups;
        MPMG_CHECK(mpmg_launch_pdl(pdl, scatter_kernel, dim3((n + keys_per_block - 1) / keys_per_block), dim3(256),
                                   0, s, keys, n, (uint32_t)ctx->ne, ctx->bin.cursor, ctx->bin.slots, ctx->perm,
                                   ctx->bin.rank, sorted_keys));
        ctx->launches += 1;
    }
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}
