// Cell sort that allocates nothing: mpmg_sort_cells_noalloc.
//
// Some callers cannot call cudaMalloc.  A host program that hands all device
// memory to its own pool allocator may forbid any other allocation, and a
// plugin that the reference's C driver dlopens (materials and boundary
// conditions) has no handle on device memory management at all.  This entry
// point serves them.  It produces the same stable element order and offsets
// as the binning every mpmg_step performs, with the LSD radix sort of
// mpmg_sort.cu, on device arrays the caller passes in and out.  Its scratch
// lives in one fixed, file-scope device array.
//
// The scratch array below is held by every GPU that loads this library, for
// the life of the process.  Its capacity is MPMG_NOALLOC_MAX_PARTICLES keys
// (2^20, the 1 048 576-particle workload; about 19 MB); larger inputs are
// rejected with MPMG_ERR_SCRATCH_LIMIT.  All calls share the one array, so
// calls that overlap on the GPU (different streams, or different host threads
// on the same device) race and must be serialised by the caller.  Nothing in
// the array must start at zero: every call rewrites the keys it sorts, the
// index sequence and the histograms it reads.
//
// Keys outside [0, num_elements] (the reference marks a particle outside the
// grid with -1) are clamped to num_elements, the outside marker, while they
// are copied into the scratch, so every key sorts into the outside run at the
// end.  The sort reads only that copy after the first kernel, so the outputs
// may not alias each other but d_sorted_keys may be d_keys itself.
#include <mutex>
#include <stdio.h>

#include "mpmg_internal.cuh"

namespace {

constexpr size_t kMaxKeys = MPMG_NOALLOC_MAX_PARTICLES;
constexpr size_t kMaxRadix = 1024;
constexpr size_t kTileKeys = 2048;
constexpr size_t kMaxTiles = (kMaxKeys + kTileKeys - 1) / kTileKeys;
// clamped keys + keys_alt + vals_alt + index sequence + per-tile histograms
// + digit totals
constexpr size_t kWords = 4 * kMaxKeys + kMaxRadix * kMaxTiles + kMaxRadix;

// In host code this name is only a host-side stand-in for the array, not a
// device address: the host passes the address cudaGetSymbolAddress returns.
static __device__ __align__(256) uint32_t g_sort_scratch[kWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t *g_scratch_addr[kMaxDevices] = {nullptr};

// The keys the sort reads: d_keys with every key outside [0, ne] replaced by
// ne; and the index sequence 0..n-1 the permutation starts from.
__global__ void clamp_iota_kernel(const int *__restrict__ keys, int n, int ne, uint32_t *__restrict__ keys_in,
                                  uint32_t *__restrict__ index)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int k = keys[i];
        keys_in[i] = (k < 0 || k > ne) ? (uint32_t)ne : (uint32_t)k;
        index[i] = (uint32_t)i;
    }
}

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
int scratch_address(uint32_t **out)
{
    int dev = 0;
    MPMG_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        mpmg_set_error("device ordinal %d beyond the %d devices the set-up tracks", dev, kMaxDevices);
        return MPMG_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return mpmg_cuda_status(e, "cudaGetSymbolAddress(sort scratch)");
        g_scratch_addr[dev] = (uint32_t *)p;
    }
    *out = g_scratch_addr[dev];
    return MPMG_OK;
}

}  // namespace

extern "C" int mpmg_sort_cells_noalloc(const int *d_keys, int n, int num_elements, int *d_sorted_keys,
                                       int *d_perm, int *d_cell_start, void *stream)
{
    if (n < 0 || num_elements < 1 || d_cell_start == nullptr ||
        (n > 0 && (d_keys == nullptr || d_sorted_keys == nullptr || d_perm == nullptr))) {
        mpmg_set_error("sort_cells_noalloc: bad arguments");
        return MPMG_ERR_INVALID;
    }
    if ((size_t)n > kMaxKeys) {
        mpmg_set_error("sort_cells_noalloc: %d keys exceed the fixed scratch capacity of %zu", n, kMaxKeys);
        return MPMG_ERR_SCRATCH_LIMIT;
    }
    if (num_elements >= (1 << 30)) {
        mpmg_set_error("sort_cells_noalloc: num_elements %d is not below 2^30", num_elements);
        return MPMG_ERR_INVALID;
    }
    uint32_t *base = nullptr;
    int rc = scratch_address(&base);
    if (rc != MPMG_OK) return rc;
    SortScratch sc;
    uint32_t *keys_in = base;
    sc.keys_alt = base + kMaxKeys;
    sc.vals_alt = base + 2 * kMaxKeys;
    uint32_t *index = base + 3 * kMaxKeys;
    sc.tile_hist = base + 4 * kMaxKeys;
    sc.digit_total = sc.tile_hist + kMaxRadix * kMaxTiles;
    sc.num_tiles = (int)((n + kTileKeys - 1) / kTileKeys);
    sc.capacity = (int)kMaxKeys;
    int bits = 1;
    while ((1ll << bits) <= (long long)num_elements) bits++;
    cudaStream_t s = (cudaStream_t)stream;
    if (n > 0) clamp_iota_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_keys, n, num_elements, keys_in, index);
    mpmg_sort_run(keys_in, index, n, num_elements, bits, sc, (uint32_t *)d_sorted_keys,
                  (uint32_t *)d_perm, d_cell_start, s);
    MPMG_CHECK(cudaGetLastError());
    return MPMG_OK;
}
