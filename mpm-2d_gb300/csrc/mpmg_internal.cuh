// Internal declarations of the mpm_gb300 library: the device context, the
// per-step parameter block that lives in device memory, and small device
// helpers shared by the kernels.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/mpm_gb300.h"

#define MPMG_TOL 1e-10          // process_usl.c:25
#define MPMG_NCOLORS 4
#define MPMG_DEPVAR 11          // particle.h:13
#define MPMG_GRAPH_CHUNK 8      // steps per replayed CUDA graph
#define MPMG_RECORD_SLOTS 4     // asynchronous step-record read-backs in flight

// Device status word bits (ctx->d_status); any nonzero value fails the step.
#define MPMG_DEV_ERR_SOLVER 0x1
#define MPMG_DEV_ERR_BOUNDS 0x2
#define MPMG_DEV_ERR_SPIN 0x4

// Step parameters updated on the device so that consecutive steps need no
// host round trip (and can be captured in a CUDA graph).
struct StepParams {
    double t;               // simulation time at the start of the current step
    double step_start_time; // job->step_start_time (0)
    double gravity;         // body force per unit mass along y used by this step's P2G
    long long step_count;   // completed steps
    // fluidity solve bookkeeping
    int solve_iters;
    int solve_converged;
    double solve_rel_resid;
};

enum Phase {
    PH_KEYS = 0,
    PH_SORT,
    PH_P2G,
    PH_GRID,
    PH_G2P,
    PH_FLUIDITY,
    PH_COUNT
};

struct SortScratch {
    uint32_t *keys_alt;
    uint32_t *vals_alt;
    uint32_t *tile_hist;   // [1024 digits][num tiles], digit-major
    uint32_t *digit_total; // [1024]
    int num_tiles;
    int capacity;          // particles
};

// Mixed-precision particle storage: four float4 records per particle, kept
// in element order and double-buffered (the G2P reads buffer `cur` and writes
// each particle to its sorted position in buffer 1 - cur):
//   A = {xl, yl, vx, vy}   B = {m, v, sxx, sxy}
//   C = {syy, ux, uy, Tzz} D = {gammap, gammadotp, pid (int bits), 0}
// The P2G reads A, B, C; the G2P reads and writes all four.
struct MixedState {
    float4 *A[2], *B[2], *C[2], *D[2];
    int cur;
    float *cell_sums;      // batches: 20 FP32 corner sums per element, value-major
    uint32_t *halo_perm;   // single simulations: 3 x np scratch orders of oversized shared tile elements
    float4 *node4;         // per node: ax, ay, vx, vy (FP32) for the gathers
    float2 *node_mass;     // per node: mass as float-float (hi, lo)
    int g2p_blocks;        // persistent G2P grid size
    int g2p_per_sm_max;    // G2P blocks of the current tile that fit on one SM
    int sms;
    int g2p_tile;          // particles a G2P tile (256 or 128)
    int p2g_variant;       // batched P2G tile (kP2GElems / kP2GStage index)
    double *export_buf;    // one FP64 particle field in caller order, for read-back
    float4 *nl_T, *nl_F;   // g_nonlocal_mu2: trial stress and bulk fluidity per stored particle
};

// A batch of independent simulations sharing one context: their particles,
// elements and nodes are concatenated (member k first at poff[k], eoff[k],
// noff[k]; each offset array has count + 1 entries), so the binning, the
// graphs and the step orchestration are those of one simulation, and the
// mixed kernels look each index's member up in the offset tables.
struct BatchInfo {
    int count;
    std::vector<mpmg_config> cfg;
    std::vector<size_t> poff, eoff, noff;
    void *d_members;       // device table of per-member constants (mpmg_mixed.cu)
    int *d_elem_off;       // eoff as int32, count + 1
    int *d_node_off;       // noff as int32, count + 1
};

// Counting-sort binning scratch (mpmg_bin.cu).  Bins 0..ne-1 count the keys
// of each element, bin ne + g the keys outside the grid at storage positions
// 32 g .. 32 g + 31.
struct BinScratch {
    uint32_t *counts;      // bins (zero between steps)
    uint32_t *cursor;      // scatter cursors (exclusive prefix of the bins)
    unsigned long long *tile_state;   // per 2048-bin tile: look-back word; then ticket and epoch
    uint32_t *slots;       // n scattered storage positions, unordered within elements
    uint32_t *rank;        // n: sorted position of each storage position
    int bins;
    int tiles;
};

struct mpmg_ctx {
    mpmg_config cfg;
    int dev;
    cudaStream_t stream;
    size_t np, nn, ne;
    int Ex, Ey;            // elements per row / column
    double inv_h;
    int key_bits;          // bits in an element key (including the inactive sentinel)

    // Derived elastic constants (the material plugins' material_init).
    double G, K, lambda;

    // Particle state, structure of arrays, caller's particle order.
    double *x, *y, *vx, *vy, *m, *v, *v0, *sxx, *sxy, *syy, *ux, *uy;
    double *Tzz;                    // g_local_mu2 out-of-plane stress
    double *state[MPMG_DEPVAR];     // allocated per material (NULL = always zero)
    double *ax, *ay, *exx, *exy, *eyy, *wxy, *xl, *yl;  // transients (store_transients)
    int *in_element;
    int *active;

    // Cell sort.
    uint32_t *keys;        // element key per particle (num_elements for inactive)
    uint32_t *sorted_keys;
    uint32_t *perm;
    int *cell_start;       // num_elements + 1
    BinScratch bin;

    // P2G per-element corner sums: 20 values per element, value-major.
    double *cell_sums;

    // Grid.
    double *node_m, *node_ax, *node_ay, *node_vx, *node_vy;
    double *node_mx, *node_my, *node_fx, *node_fy;   // store_transients
    double *node_gf;

    // Nonlocal fluidity solve.
    double *elem_k;        // 10 matrix entries per element, value-major
    double *elem_f;        // 4 RHS entries per element, value-major
    double *nl_trial;      // g_nonlocal_mu2: trial stress from the G2P, 5 per particle, value-major
    double *cg_x, *cg_r, *cg_p, *cg_q, *cg_dinv, *cg_w;   // per node
    double *cg_coef;       // 9-point rows of the assembled matrix, 9 per node
    double *cg_partials;   // per-block partial sums
    unsigned int *cg_barrier;  // grid barrier counter + generation
    int cg_blocks;
    int cg_tile_blocks;    // pcg_tile_kernel: blocks (0: the grid does not fit, pcg_kernel runs)
    int cg_tile_nodes;     // pcg_tile_kernel: nodes per block
    size_t cg_tile_smem;   // pcg_tile_kernel: dynamic shared memory per block
    // multigrid-preconditioned solve (pcg_mg_kernel): level table on the host
    // and its device copy (NULL when the grid does not fit the kernel), pools
    struct MgPlan *mg_host, *mg_dev;
    float *mg_rows;
    unsigned long long *mg_words;
    unsigned int *mg_tag;
    size_t mg_smem;

    StepParams *d_params;  // one record per simulation (a batch holds several)
    StepParams h_params;   // host mirror of the first, refreshed on read-back
    int *d_status;
    unsigned char *h_record;   // pinned host mirror of the step records and status
    // asynchronous read-backs of the step records (mpmg_record_async): pinned
    // ring slots, each completed by its event
    unsigned char *h_ring[MPMG_RECORD_SLOTS];
    cudaEvent_t ring_ev[MPMG_RECORD_SLOTS];
    // per-step records written by the step itself into mapped pinned memory
    // (mpmg_record_ring): slot k holds a step number (8 bytes, written last)
    // and then the step record
    unsigned char *rring_h;
    unsigned char *rring_d;
    int rring_slots;
    size_t rring_slot_bytes;
    size_t status_offset;      // byte offset of the status word in the record block

    // Batched ensemble (mpmg_batch_create): several independent simulations
    // in one context, NULL for a single simulation.
    BatchInfo *batch;

    // Tape of the last mpmg_adj_forward_tape run (mpmg_adjoint.cu).
    struct AdjTape *adj;

    // Mixed precision (cfg.precision == MPMG_PRECISION_MIXED).
    MixedState *mixed;

    // CUDA graphs of whole steps (index: buffer parity of the mixed form):
    // a chunk of graph_steps steps and a single step, captured on first use.
    int graph_steps;       // MPMG_GRAPH_CHUNK unless tuned (mpmg_autotune)
    cudaGraphExec_t graph_chunk[2];
    cudaGraphExec_t graph_single[2];
    long graph_chunk_launches[2];
    long graph_single_launches[2];

    // Timing.
    int timing;
    int phase_used[PH_COUNT];
    cudaEvent_t ev[2 * PH_COUNT];
    double phase_ms[PH_COUNT];
    long phase_launches[PH_COUNT];
    long launches;
};

// Bit casts usable in host code (particle ids travel in float4 records).
static inline int mpmg_float_bits(float f)
{
    int i;
    memcpy(&i, &f, sizeof(i));
    return i;
}

static inline float mpmg_bits_float(int i)
{
    float f;
    memcpy(&f, &i, sizeof(f));
    return f;
}

// Error helpers (host).
void mpmg_set_error(const char *fmt, ...);
int mpmg_cuda_status(cudaError_t e, const char *what);

#define MPMG_CHECK(call)                                          \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return mpmg_cuda_status(_e, #call); \
    } while (0)

// Kernel launch helpers implemented per translation unit.
// Scratch words (uint32) a sort of n keys needs, and its tile count.
size_t mpmg_sort_scratch_words(size_t n, int key_bits, int *num_tiles_out);
// Sort with caller-provided scratch; returns the number of launches issued.
int mpmg_sort_run(const uint32_t *keys, const uint32_t *vals, int n, int ne, int key_bits,
                  const SortScratch &sc, uint32_t *sorted_keys, uint32_t *perm, int *cell_start,
                  cudaStream_t s);
int mpmg_launch_step(mpmg_ctx *ctx);             // one full step
int mpmg_bin_init(mpmg_ctx *ctx);
void mpmg_bin_free(mpmg_ctx *ctx);
// Stand-alone count of keys[n] (<= ne) into the bins.
int mpmg_bin_count(mpmg_ctx *ctx, const uint32_t *keys);
// Scan of the counted bins and scatter: cell_start, sorted_keys (unless
// null), and perm for keys outside the grid; element slots stay unordered in
// bin.slots until a P2G kernel orders them into perm (mpmg_order_segment).
// mpmg_bin_reset restores the look-back state after a timed-out wait.
int mpmg_bin_scan_scatter(mpmg_ctx *ctx, const uint32_t *keys, uint32_t *sorted_keys, bool pdl = false);
int mpmg_bin_reset(mpmg_ctx *ctx);
int mpmg_nonlocal_init(mpmg_ctx *ctx);
void mpmg_nonlocal_free(mpmg_ctx *ctx);
int mpmg_launch_fluidity(mpmg_ctx *ctx);         // nonlocal: assembly, solve, stress
int mpmg_launch_solve(mpmg_ctx *ctx);            // nonlocal: the fluidity PCG alone
int mpmg_solve_fluidity_system(mpmg_ctx *ctx, const double *elem_k, const double *elem_f, const double *node_m,
                               const int *cell_start, double *x, bool zero_start);
int mpmg_launch_material_only(mpmg_ctx *ctx);
int mpmg_mixed_init(mpmg_ctx *ctx, const double *m, const double *v, const double *x, const double *y,
                    const double *vx, const double *vy, const double *sxx, const double *sxy,
                    const double *syy);
void mpmg_mixed_free(mpmg_ctx *ctx);
int mpmg_mixed_set_g2p_per_sm(mpmg_ctx *ctx, int per_sm);   // returns the value set
int mpmg_mixed_set_tiles(mpmg_ctx *ctx, int p2g_variant, int g2p_tile);
int mpmg_mixed_p2g_variants();
void mpmg_mixed_p2g_shape(int v, int *elements, int *stage);
int mpmg_mixed_step(mpmg_ctx *ctx);
// Host read-back / write of a mixed particle or node field; returns
// MPMG_ERR_UNKNOWN_FIELD for names the mixed state does not hold.
int mpmg_mixed_get(mpmg_ctx *ctx, const char *name, double *out);
int mpmg_mixed_set(mpmg_ctx *ctx, const char *name, const double *in);
int mpmg_mixed_get_many(mpmg_ctx *ctx, int count, const char *const *names, double *const *out, bool *done);
int mpmg_mixed_get_map(mpmg_ctx *ctx, int *in_element, int *active);
void mpmg_adj_free(mpmg_ctx *ctx);

void mpmg_phase_begin(mpmg_ctx *ctx, int phase);
void mpmg_phase_end(mpmg_ctx *ctx, int phase);

// ---------------------------------------------------------------------------
// Device helpers.

// Element containing (xp, yp), bit-exact with WHICH_ELEMENT4
// (process_usl.c:43-44): e = (int)(floor(x/h) + floor(y/h) * (Nx - 1)) when
// 0 <= x < xmax and 0 <= y < ymax, else -1.  x * (1/h) replaces the division
// unless the quotient is within a relative 2^-44 of an integer, where the
// correctly rounded division decides (both products are within 2^-51
// relative of x/h).  Out-of-range results (x/h rounding up to Nx-1 just below
// xmax) are reported as -1.
__device__ __forceinline__ int mpmg_which_element(double xp, double yp, double h, double inv_h,
                                                  double xmax, double ymax, int Ex, int Ey)
{
    if (!(xp < xmax && xp >= 0.0 && yp < ymax && yp >= 0.0)) return -1;
    double qx = xp * inv_h;
    double fx = floor(qx);
    double rx = qx - fx;
    if (rx < 0x1p-44 * (qx + 1.0) || (1.0 - rx) < 0x1p-44 * (qx + 1.0)) fx = floor(__ddiv_rn(xp, h));
    double qy = yp * inv_h;
    double fy = floor(qy);
    double ry = qy - fy;
    if (ry < 0x1p-44 * (qy + 1.0) || (1.0 - ry) < 0x1p-44 * (qy + 1.0)) fy = floor(__ddiv_rn(yp, h));
    if (fx >= (double)Ex || fy >= (double)Ey) return -1;
    return (int)(fx + fy * (double)Ex);
}

// floor(x / h) in integer and FP32 arithmetic, or -1 where that cannot
// decide it.  x >= 2^-126 (else -1).  The FP32 value of x taken from the top
// 20 mantissa bits (relative error below 2^-20) times inv_hf = RN32(1 / h)
// lies within q * 2^-19.8 of x / h; where it is farther than
// q * 2^-19 + 2^-22 from every integer, x / h, its FP64 product and its FP64
// quotient all floor to the same integer, which is returned.
__device__ __forceinline__ int mpmg_floor_quotient_fast(double x, float inv_hf)
{
    const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
    if (hi < (897u << 20) || hi >= (1151u << 20)) return -1;
    const float xf = __uint_as_float((hi - (896u << 20)) << 3);
    const float q = xf * inv_hf;
    const float fl = floorf(q);
    const float fr = q - fl;
    const float margin = fmaf(q, 0x1p-19f, 0x1p-22f);
    if (!(fr > margin && fr < 1.0f - margin) || q >= 0x1p22f) return -1;
    return (int)fl;
}

// mpmg_which_element with the common case in integer and FP32 arithmetic:
// the range test on the bit patterns (non-negative doubles order as
// integers; -0.0 counts as inside, NaN as outside) and each floor from
// mpmg_floor_quotient_fast; a coordinate that lands near an element edge
// takes mpmg_which_element.  The result equals mpmg_which_element's for every
// input.  xmax_bits, ymax_bits are the bit patterns of the (positive) bounds.
__device__ __forceinline__ int mpmg_which_element_fast(double xp, double yp, double h, double inv_h,
                                                       float inv_hf, double xmax, double ymax,
                                                       long long xmax_bits, long long ymax_bits, int Ex, int Ey)
{
    const long long bx = __double_as_longlong(xp), by = __double_as_longlong(yp);
    const long long mag = 0x7fffffffffffffffLL;
    const bool in_x = (bx >= 0 || bx == (long long)0x8000000000000000ULL) && (bx & mag) < xmax_bits;
    const bool in_y = (by >= 0 || by == (long long)0x8000000000000000ULL) && (by & mag) < ymax_bits;
    if (!(in_x && in_y)) return -1;
    const int fx = mpmg_floor_quotient_fast(xp, inv_hf);
    const int fy = mpmg_floor_quotient_fast(yp, inv_hf);
    if (fx < 0 || fy < 0) return mpmg_which_element(xp, yp, h, inv_h, xmax, ymax, Ex, Ey);
    if (fx >= Ex || fy >= Ey) return -1;
    return fx + fy * Ex;
}

// Local coordinates in the element with bottom-left node at (xn, yn), with
// the reference's snap to +-1 within 1e-10 (particle.c:14-30).
// |xl| > 1 is tested on the bit pattern (positive doubles order as
// integers), so that the common case costs no FP64 compare.
__device__ __forceinline__ double mpmg_local_coord(double xp, double xn, double inv_h)
{
    double xl = (xp - xn) * inv_h;
    if ((__double_as_longlong(xl) & 0x7fffffffffffffffLL) > 0x3ff0000000000000LL) {
        double sg = copysign(1.0, xl);
        if (((sg * xl) - 1.0) < MPMG_TOL) xl = sg;
    }
    return xl;
}

// The same with xl = x / h - c in one FMA from the element's column (or row)
// c (one FP64 operation in place of three; xl differs from (x - c h) / h by
// a few ulps of x / h, about 1e-14 on a 512-element grid).
__device__ __forceinline__ double mpmg_local_coord_fma(double xp, double c, double inv_h)
{
    double xl = fma(xp, inv_h, -c);
    if ((__double_as_longlong(xl) & 0x7fffffffffffffffLL) > 0x3ff0000000000000LL) {
        double sg = copysign(1.0, xl);
        if (((sg * xl) - 1.0) < MPMG_TOL) xl = sg;
    }
    return xl;
}

// Counts one key into the bins (see BinScratch): bins[key] for keys inside
// the grid, bins[sentinel + group] for keys outside it, where group is the
// key's destination position / 32.  Runs of equal bins in consecutive lanes
// are aggregated into one atomic (the keys arrive nearly sorted, so a warp
// holds a few runs).  Every lane of the warp must call it (valid marks lanes
// that carry a key).
__device__ __forceinline__ void mpmg_bin_count(uint32_t key, bool valid, uint32_t sentinel, uint32_t group,
                                               uint32_t *bins)
{
    const int lane = threadIdx.x & 31;
    const uint32_t bin = valid ? ((key == sentinel) ? sentinel + group : key) : 0xffffffffu;
    const uint32_t prev = __shfl_up_sync(0xffffffffu, bin, 1);
    const bool start = valid && (lane == 0 || prev != bin);
    const uint32_t starts = __ballot_sync(0xffffffffu, start);
    const uint32_t invalid = ~__ballot_sync(0xffffffffu, valid);
    if (start) {
        const uint32_t above = lane == 31 ? 0u : (starts | invalid) & (0xfffffffeu << lane);
        const int end = above ? __ffs(above) - 1 : 32;
        atomicAdd(&bins[bin], (uint32_t)(end - lane));
    }
}

__device__ __forceinline__ uint32_t mpmg_smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Programmatic dependent launch.  A kernel launched with
// mpmg_launch_pdl may start while the kernel before it in the stream is
// still running; mpmg_pdl_wait blocks until that kernel has completed and
// its writes are visible (a no-op for an ordinary launch), and
// mpmg_pdl_trigger lets the next kernel start launching.  Every kernel of the
// mixed step triggers only after its own wait, so when a kernel starts, the
// kernel two places before it has completed: data written by that kernel or
// earlier ones may be read before the wait, data of the immediately
// preceding kernel only after it.
__device__ __forceinline__ void mpmg_pdl_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void mpmg_pdl_trigger()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t mpmg_launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                   cudaStream_t stream, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, ((KArgs)args)...);
}

// Asynchronous global -> shared copies of 16 or 4 bytes (cp.async, cached in
// L1), completed by mpmg_cp_async_wait_all.
__device__ __forceinline__ void mpmg_cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(mpmg_smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void mpmg_cp_async4(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(mpmg_smem_addr(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void mpmg_cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Unsigned division by a run-time constant d >= 1 (Granlund and Montgomery,
// "Division by invariant integers using multiplication", 1994, round-up
// variant): n / d = (umulhi(n, magic) + n) >> shift for every 32-bit n, with
// shift = ceil(log2 d) and magic = floor(2^32 (2^shift - d) / d) + 1.
struct MpmgDiv {
    uint32_t magic, shift, d;
};

inline MpmgDiv mpmg_div_init(uint32_t d)
{
    MpmgDiv v;
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < (unsigned long long)d) l++;
    v.magic = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / d) + 1ull);
    v.shift = l;
    v.d = d;
    return v;
}

__device__ __forceinline__ uint32_t mpmg_div(uint32_t n, const MpmgDiv &v)
{
    return (uint32_t)(((unsigned long long)__umulhi(n, v.magic) + n) >> v.shift);
}

// Bulk asynchronous copies (TMA, cp.async.bulk) into shared memory, completed
// on an mbarrier, and the bounded wait for them.
__device__ __forceinline__ void mpmg_mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mpmg_smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mpmg_mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier shared-memory accesses before later
// asynchronous-proxy (bulk copy) accesses.
__device__ __forceinline__ void mpmg_fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mpmg_mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mpmg_smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// dst, src and bytes must be multiples of 16 bytes.
__device__ __forceinline__ void mpmg_bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     mpmg_smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(mpmg_smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mpmg_mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(mpmg_smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for phase `parity` of the barrier to complete; false after `limit`
// polls.
__device__ __forceinline__ bool mpmg_mbar_wait(uint64_t *bar, uint32_t parity, long long limit)
{
    for (long long polls = 0; polls < limit; polls++)
        if (mpmg_mbar_try_wait(bar, parity)) return true;
    return false;
}

// perm[k0..k1) = slots[k0..k1) in ascending order (insertion sort: elements
// hold a handful of particles), and rank[perm[k]] = k when rank is given.
__device__ __forceinline__ void mpmg_order_segment(const uint32_t *__restrict__ slots, uint32_t *__restrict__ perm,
                                                   uint32_t *__restrict__ rank, int k0, int k1)
{
    for (int j = k0; j < k1; j++) {
        const uint32_t x = slots[j];
        int i = j - 1;
        while (i >= k0 && perm[i] > x) {
            perm[i + 1] = perm[i];
            i--;
        }
        perm[i + 1] = x;
    }
    if (rank != nullptr)
        for (int j = k0; j < k1; j++) rank[perm[j]] = (uint32_t)j;
}

// Grid barrier over all blocks of a cooperative launch.  Every wait is
// bounded: after `limit` polls the barrier sets MPMG_DEV_ERR_SPIN in *status
// and returns false, and the caller leaves the kernel.
__device__ __forceinline__ bool mpmg_grid_barrier(unsigned int *bar, unsigned int nblocks,
                                                  int *status, long long limit)
{
    __syncthreads();
    bool ok = true;
    if (threadIdx.x == 0) {
        volatile unsigned int *gen = bar + 1;
        unsigned int g = *gen;
        __threadfence();
        unsigned int arrived = atomicAdd(bar, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long polls = 0;
            while (*gen == g) {
                if (++polls > limit || (*(volatile int *)status & MPMG_DEV_ERR_SPIN) != 0) {
                    atomicOr(status, MPMG_DEV_ERR_SPIN);
                    ok = false;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok && (*(volatile int *)status & MPMG_DEV_ERR_SPIN) == 0;
}
