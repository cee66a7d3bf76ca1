// Stable LSD radix sort of (element key, particle index) pairs, and the
// per-element start offsets of the sorted order.  The allocation-free entry
// point (mpmg_sort_noalloc.cu) runs it on its fixed scratch; the step bins
// particles with the counting sort of mpmg_bin.cu, which gives the same
// order.
//
// The reference groups particles by element in find_filled_elements
// (libmpm/process_usl.c:677-723): for each element, its particles in
// ascending particle index.  A stable sort of the keys over particle indices
// 0..n-1 reproduces exactly those groups, so the permutation is bit-exact
// against the reference's lists.
//
// Keys need ceil(log2(num_elements + 1)) bits (18 for 512^2 elements); they
// are sorted in ceil(bits / 10) passes of at most 10 bits.  Each pass:
//   upsweep    per-tile digit histogram (tile = 2048 keys, shared atomics)
//   scan       one warp per digit: exclusive prefix of that digit's counts
//              over the tiles, and the digit's total
//   downsweep  every warp ranks its 256 contiguous keys stably (match_any +
//              a warp-private digit histogram), the block turns the per-warp
//              counts into offsets (digit prefix over the whole input + this
//              tile's prefix + earlier warps), and keys and values scatter
// Integer-only and deterministic for any launch order.
#include "mpmg_internal.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRounds = 8;                       // keys per lane
constexpr int kTile = kThreads * kRounds;        // 2048 keys per block
constexpr int kMaxBits = 10;
constexpr int kMaxRadix = 1 << kMaxBits;

__global__ void __launch_bounds__(kThreads) upsweep_kernel(const uint32_t *__restrict__ keys, int n,
                                                           int shift, int bits, int num_tiles,
                                                           uint32_t *__restrict__ tile_hist)
{
    __shared__ uint32_t hist[kMaxRadix];
    const int radix = 1 << bits;
    for (int d = threadIdx.x; d < radix; d += kThreads) hist[d] = 0;
    __syncthreads();
    const uint32_t mask = (uint32_t)radix - 1u;
    const int base = blockIdx.x * kTile;
#pragma unroll
    for (int k = 0; k < kRounds; k++) {
        int idx = base + k * kThreads + threadIdx.x;
        if (idx < n) atomicAdd(&hist[(keys[idx] >> shift) & mask], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < radix; d += kThreads)
        tile_hist[(size_t)d * num_tiles + blockIdx.x] = hist[d];
}

// One warp per digit: exclusive scan of tile_hist[d][0..num_tiles) in place,
// total of digit d into digit_total[d].
__global__ void __launch_bounds__(kThreads) scan_tiles_kernel(uint32_t *__restrict__ tile_hist,
                                                              int num_tiles, int radix,
                                                              uint32_t *__restrict__ digit_total)
{
    const int lane = threadIdx.x & 31;
    const int d = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (d >= radix) return;
    uint32_t *row = tile_hist + (size_t)d * num_tiles;
    uint32_t run = 0;
    for (int base = 0; base < num_tiles; base += 32) {
        int t = base + lane;
        uint32_t v = (t < num_tiles) ? row[t] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += u;
        }
        if (t < num_tiles) row[t] = run + incl - v;
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) digit_total[d] = run;
}

__global__ void __launch_bounds__(kThreads) downsweep_kernel(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in, int n, int shift,
    int bits, int num_tiles, const uint32_t *__restrict__ tile_prefix,
    const uint32_t *__restrict__ digit_total, uint32_t *__restrict__ keys_out,
    uint32_t *__restrict__ vals_out)
{
    __shared__ uint32_t warp_hist[kWarps][kMaxRadix];   // counts, then per-warp bases
    __shared__ uint32_t digit_base[kMaxRadix];
    __shared__ uint32_t warp_sums[kWarps];
    const int radix = 1 << bits;
    const uint32_t mask = (uint32_t)radix - 1u;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;

    for (int k = threadIdx.x; k < kWarps * kMaxRadix; k += kThreads) (&warp_hist[0][0])[k] = 0;

    // Exclusive prefix of the digit totals (the digit's start in the output).
    {
        const int per = kMaxRadix / kThreads;            // 4 digits per thread
        uint32_t local[per];
        uint32_t s = 0;
#pragma unroll
        for (int j = 0; j < per; j++) {
            int d = threadIdx.x * per + j;
            local[j] = (d < radix) ? digit_total[d] : 0u;
            s += local[j];
        }
        uint32_t incl = s;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t u = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += u;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        uint32_t wbase = 0;
        for (int w = 0; w < warp; w++) wbase += warp_sums[w];
        uint32_t run = wbase + incl - s;
#pragma unroll
        for (int j = 0; j < per; j++) {
            int d = threadIdx.x * per + j;
            if (d < radix) digit_base[d] = run + tile_prefix[(size_t)d * num_tiles + blockIdx.x];
            run += local[j];
        }
    }
    __syncthreads();

    // Each warp ranks its contiguous 256 keys in order (stable).
    const int wbase_idx = blockIdx.x * kTile + warp * (kRounds * 32);
    uint32_t key[kRounds], val[kRounds], rank[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
        const int idx = wbase_idx + r * 32 + lane;
        const bool valid = idx < n;
        key[r] = valid ? keys_in[idx] : 0xffffffffu;
        val[r] = valid ? vals_in[idx] : 0u;
        const uint32_t d = (key[r] >> shift) & mask;
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 0xffffffffu) & vmask;
        uint32_t before = 0;
        if (valid) before = warp_hist[warp][d];
        __syncwarp();
        rank[r] = before + __popc(peers & lt_mask);
        if (valid && (peers & lt_mask) == 0) warp_hist[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // Per digit: exclusive prefix over warps, offset by the digit's base.
    for (int d = threadIdx.x; d < radix; d += kThreads) {
        uint32_t run = digit_base[d];
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
            uint32_t c = warp_hist[w][d];
            warp_hist[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
        const int idx = wbase_idx + r * 32 + lane;
        if (idx < n) {
            const uint32_t d = (key[r] >> shift) & mask;
            const uint32_t dst = warp_hist[warp][d] + rank[r];
            keys_out[dst] = key[r];
            vals_out[dst] = val[r];
        }
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

size_t mpmg_sort_scratch_words(size_t n, int key_bits, int *num_tiles_out)
{
    int tiles = (int)((n + kTile - 1) / kTile);
    if (tiles < 1) tiles = 1;
    if (num_tiles_out) *num_tiles_out = tiles;
    (void)key_bits;
    // keys_alt + vals_alt + tile histogram + digit totals
    return 2 * (n > 0 ? n : 1) + (size_t)kMaxRadix * tiles + kMaxRadix;
}

// Sorts keys/vals (n entries, keys < 2^key_bits) into sorted_keys/perm using
// the given scratch, then fills cell_start[0..ne].  Returns launches issued.
int mpmg_sort_run(const uint32_t *keys, const uint32_t *vals, int n, int ne, int key_bits,
                  const SortScratch &sc, uint32_t *sorted_keys, uint32_t *perm, int *cell_start,
                  cudaStream_t s)
{
    int launches = 0;
    if (n > 0) {
        const int passes = (key_bits + kMaxBits - 1) / kMaxBits;
        const int base_bits = key_bits / passes, extra = key_bits % passes;
        const int tiles = (n + kTile - 1) / kTile;
        const uint32_t *src_k = keys, *src_v = vals;
        int shift = 0;
        for (int p = 0; p < passes; p++) {
            const int bits = base_bits + (p < extra ? 1 : 0);
            const int radix = 1 << bits;
            const bool to_out = ((passes - 1 - p) % 2) == 0;
            uint32_t *dst_k = to_out ? sorted_keys : sc.keys_alt;
            uint32_t *dst_v = to_out ? perm : sc.vals_alt;
            upsweep_kernel<<<tiles, kThreads, 0, s>>>(src_k, n, shift, bits, tiles, sc.tile_hist);
            scan_tiles_kernel<<<(radix + kWarps - 1) / kWarps, kThreads, 0, s>>>(sc.tile_hist, tiles, radix,
                                                                                sc.digit_total);
            downsweep_kernel<<<tiles, kThreads, 0, s>>>(src_k, src_v, n, shift, bits, tiles, sc.tile_hist,
                                                        sc.digit_total, dst_k, dst_v);
            launches += 3;
            src_k = dst_k;
            src_v = dst_v;
            shift += bits;
        }
    }
    cell_start_kernel<<<(ne + 1 + 255) / 256, 256, 0, s>>>(sorted_keys, n, ne, cell_start);
    return launches + 1;
}
