// Allocation-free grid solve: uastar_grid_solve_noalloc.
//
// Who needs this: code that may not call cudaMalloc/cudaFree while it runs —
// a host inside a CUDA-graph-captured or real-time loop, a plugin living in
// another framework's memory pool, an allocator-free embedded service.  The
// regular engine owns grow-on-demand device buffers and may reallocate them
// on any call; this entry point instead runs the same GA* search kernel
// (ga_search on a whole-grid team) out of one fixed device array that the
// library reserves at load time, so a call allocates nothing.
//
// Costs and limits of that choice:
//   - every GPU that loads the library holds kScratchBytes (about 53 MB)
//     of device memory until the process exits;
//   - grids are limited to kMaxCells cells; the search itself is limited to
//     kTableSlots * 0.8 dedup slots and kHeaps heaps of kHeapCap entries
//     (an instance that needs more reports UASTAR_HASH_FULL or
//     UASTAR_HEAP_OVERFLOW in its result);
//   - all calls share the one array: two calls whose work overlaps on the
//     GPU (different streams, or different host threads) race and corrupt
//     each other; serialize them;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress); make that first call outside any stream
//     capture.  The address is kept for the life of the process: after a
//     cudaDeviceReset the array lives in a new context and this entry point
//     must not be called again in that process;
//   - every team-barrier wait of the search gives up after 10 s and the
//     result then reports UASTAR_TIMEOUT;
//   - a call that returns anything but UASTAR_OK queued nothing that writes
//     the result record (its contents are unchanged); an error left pending
//     by the caller's earlier CUDA work is reported as UASTAR_CUDA_ERROR and
//     left pending, before anything is queued.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/uastar_gpu.h"
#include "ga_device.cuh"
#include "ga_problems.cuh"
#include "ga_search.cuh"

using namespace uastar;

namespace {

constexpr uint32_t kBlock = 256;                 // threads per CTA
constexpr uint32_t kHeapsPerCta = 64;            // 4 threads per heap
constexpr uint32_t kCtas = 4;
constexpr uint32_t kHeaps = kCtas * kHeapsPerCta;
constexpr uint32_t kTopLevels = 6;               // heap levels in shared memory
constexpr uint32_t kHeapCap = 4095;              // entries per heap
constexpr uint32_t kTableLog2 = 20;              // dedup slots
constexpr uint64_t kTableSlots = 1ull << kTableLog2;
constexpr uint64_t kMaxCells = 1ull << 22;       // largest grid accepted (e.g. 2048 x 2048)

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
// heap block per heap: saved top (64 entries) + 576 bricks of 8 entries
// (heap_geometry<GridProblem>(6, 4095) = {4672, 4095}, checked at set-up)
constexpr uint32_t kHeapStride = 4672;
constexpr size_t kOffState = 0;
constexpr size_t kOffSizes = align256(kOffState + sizeof(TeamState));
constexpr size_t kOffCand = align256(kOffSizes + kHeaps * sizeof(uint32_t));
constexpr size_t kOffHeaps = align256(kOffCand + cand_records<GridProblem>(kCtas, kHeapsPerCta) * sizeof(Cand));
constexpr size_t kOffTable = align256(kOffHeaps + (size_t)kHeaps * kHeapStride * sizeof(GridEntry));
constexpr size_t kScratchBytes = align256(kOffTable + kTableSlots * sizeof(Slot));

// The only device memory this entry point uses besides the caller's buffers.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Per-device address of g_noalloc_scratch (looked up once per device).
constexpr int kMaxDevices = 64;
unsigned char *g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_setup_mu;

__global__ void k_noalloc_reset(unsigned char *scratch) {
    // team state: everything zero except the "unset" costs and statuses
    TeamState *st = reinterpret_cast<TeamState *>(scratch + kOffState);
    uint32_t *sizes = reinterpret_cast<uint32_t *>(scratch + kOffSizes);
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) team_state_init(st);
    for (uint32_t i = t; i < kHeaps; i += gridDim.x * blockDim.x) sizes[i] = 0;
    // dedup table: every slot empty (key and g all ones, prev = none)
    uint4 *tab = reinterpret_cast<uint4 *>(scratch + kOffTable);
    const uint4 ff = make_uint4(~0u, ~0u, ~0u, ~0u);
    for (uint64_t i = t; i < kTableSlots * 2; i += (uint64_t)gridDim.x * blockDim.x) tab[i] = ff;
}

__global__ void __launch_bounds__(kBlock, 1) k_noalloc_search(GridProblem prob, SearchMem<GridEntry> m,
                                                              TeamState *st, uint64_t timeout_ns) {
    extern __shared__ __align__(128) unsigned char smem[];
    GridTeam team{st, 0u, timeout_ns};
    ga_search<GridProblem>(prob, team, m, kHeapsPerCta, smem, ~0ull);
}

// Result + path, walking prev pointers from the goal (one thread), then
// reversing the path in place to run start -> goal.
__global__ void k_noalloc_finish(const unsigned char *scratch, int32_t *path, int64_t cap,
                                 uastar_noalloc_grid_result *out) {
    const TeamState *st = reinterpret_cast<const TeamState *>(scratch + kOffState);
    const Slot *tab = reinterpret_cast<const Slot *>(scratch + kOffTable);
    __shared__ long long s_len;
    if (threadIdx.x == 0) {
        uastar_noalloc_grid_result r;
        memset(&r, 0, sizeof r);
        r.status = (int32_t)__ldcg(&st->status);
        r.expanded = (int64_t)__ldcg(&st->expanded);
        r.generated = (int64_t)__ldcg(&st->generated);
        r.rounds = (int64_t)__ldcg(&st->round);
        long long n = 0;
        if (r.status == ST_OK) {
            const unsigned long long gbest = __ldcg(&st->goal_best);
            r.straight = (int64_t)(gbest >> 32);
            r.diagonal = (int64_t)(gbest & 0xffffffffu);
            uint32_t s = __ldcg(&st->goal_slot);
            while (s != kNone && n < cap) {
                uint64_t key;
                uint32_t prev;
                slot_key_prev(tab + s, GridProblem::kLink, key, prev);
                path[n++] = (int32_t)key;
                s = prev;
            }
            if (s != kNone) {
                r.status = UASTAR_ARENA_FULL;  // the caller's path buffer is too small
                n = 0;
            }
        }
        r.path_len = n;
        *out = r;
        s_len = n;
    }
    __syncthreads();
    const long long n = s_len;
    for (long long i = threadIdx.x; i < n / 2; i += blockDim.x) {
        const int32_t a = path[i], b = path[n - 1 - i];
        path[i] = b;
        path[n - 1 - i] = a;
    }
}

}  // namespace

extern "C" int32_t uastar_grid_solve_noalloc(const uint64_t *d_words, int32_t H, int32_t W, int32_t sx,
                                             int32_t sy, int32_t ex, int32_t ey, int32_t *d_path,
                                             int64_t path_cap, uastar_noalloc_grid_result *d_result,
                                             void *stream) {
    if (!d_words || !d_path || !d_result || path_cap < 1 || H <= 0 || W <= 0) return UASTAR_BAD_INPUT;
    if ((uint64_t)H * (uint64_t)W > kMaxCells) return UASTAR_BAD_INPUT;  // beyond the fixed scratch's maximum
    if (sx < 0 || sx >= H || sy < 0 || sy >= W || ex < 0 || ex >= H || ey < 0 || ey >= W) return UASTAR_BAD_INPUT;
    // an error from the caller's earlier work is theirs: report it, keep it
    if (cudaPeekAtLastError() != cudaSuccess) return UASTAR_CUDA_ERROR;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return UASTAR_CUDA_ERROR;

    // Set-up, once per device with that device current: the host-side name
    // g_noalloc_scratch is only a stand-in, the kernels need the device address.
    unsigned char *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_scratch_ptr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return UASTAR_CUDA_ERROR;
            const size_t smem = SearchSmem<GridProblem>::bytes(kHeapsPerCta, kTopLevels);
            if (cudaFuncSetAttribute(k_noalloc_search, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess)
                return UASTAR_CUDA_ERROR;
            const HeapGeometry<GridProblem> hg = heap_geometry<GridProblem>(kTopLevels, kHeapCap);
            if (hg.stride != kHeapStride) return UASTAR_CUDA_ERROR;  // layout constants out of date
            g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
        }
        scratch = g_scratch_ptr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    k_noalloc_reset<<<256, 256, 0, s>>>(scratch);
    if (cudaGetLastError() != cudaSuccess) return UASTAR_CUDA_ERROR;

    GridProblem prob;
    prob.bm = reinterpret_cast<const uint32_t *>(d_words);
    prob.H = H;
    prob.W = W;
    prob.sx = sx;
    prob.sy = sy;
    prob.ex = ex;
    prob.ey = ey;
    SearchMem<GridEntry> m;
    m.tab = reinterpret_cast<Slot *>(scratch + kOffTable);
    m.mask = kTableSlots - 1;
    m.max_inserted = (uint64_t)(kTableSlots * 0.8);
    m.max_probe = 4096;
    m.heaps = reinterpret_cast<GridEntry *>(scratch + kOffHeaps);
    m.stride = kHeapStride;
    m.hcap = kHeapCap;
    m.L = kTopLevels;
    m.heap_size = reinterpret_cast<uint32_t *>(scratch + kOffSizes);
    m.cand = reinterpret_cast<Cand *>(scratch + kOffCand);
    m.max_rounds = 1ull << 31;
    TeamState *st = reinterpret_cast<TeamState *>(scratch + kOffState);
    uint64_t timeout_ns = 10ull * 1000000000ull;  // bound on every team-barrier wait (UASTAR_TIMEOUT)
    void *args[] = {&prob, &m, &st, &timeout_ns};
    const size_t smem = SearchSmem<GridProblem>::bytes(kHeapsPerCta, kTopLevels);
    if (cudaLaunchCooperativeKernel((const void *)k_noalloc_search, dim3(kCtas), dim3(kBlock), args, smem, s) !=
        cudaSuccess)
        return UASTAR_CUDA_ERROR;
    k_noalloc_finish<<<1, 256, 0, s>>>(scratch, d_path, path_cap, d_result);
    return cudaGetLastError() == cudaSuccess ? UASTAR_OK : UASTAR_CUDA_ERROR;
}
