// kgpu_noalloc.cu — kgpu_check_edges_noalloc: the planner edge check without
// any allocation at call time.
//
// Who needs it: callers that may not allocate device memory while they run —
// a real-time planning or control loop, where cudaMalloc's implicit device
// synchronisation and unbounded latency are not acceptable, or a host
// application that reserves the device's memory up front through its own
// pool and forbids further driver allocations.  The regular entry point
// (kgpu_check_edges) grows its permutation table on demand; this variant
// instead works entirely inside one fixed, file-scope device array.
//
// The array (kNoAllocBytes, 32 MiB) holds the work-queue heads, the edge
// ordering tables for at most KGPU_NOALLOC_MAX_EDGES edges, the list of
// triangle pairs left to the FP64 re-test (65,536 entries; a longer list
// makes a fallback pass re-check every step, so results stay exact), and
// per-warp regions (FP64 link transforms + a 1,024-entry traversal spill
// stack) for up to 2,560 warps: the world's blocks per SM on GPUs of up to
// 160 SMs at two 8-warp blocks per SM (GB300: 152 SMs).  A world tuned for
// more resident blocks per SM runs here with as many as the array serves.
// Every GPU that loads the library keeps this array until the process exits.
//
// Set-up: kgpu_world_create, with the world's device current, looks up the
// array's device address with cudaGetSymbolAddress (a host variable name is
// not a device address; the lookup also loads the module that holds the
// array, which allocates it) and caches it per device, so the entry point
// itself neither loads nor allocates anything.  A call on a device where no
// world was created does that look-up itself on its first call; make that
// first call before any stream capture.  All calls share the array, and each
// call clears what must start at zero (queue heads, histogram, counters) on
// its stream, so calls that overlap on the GPU — on different streams, or
// from several host threads — race on the array and must be serialised by
// the caller.
#include <mutex>

#include "kgpu_internal.h"

namespace kgpu {
kgpu_status record_error(kgpu_status code, const char* msg);
int engine_warps_per_block();
int engine_scratch_doubles();
}  // namespace kgpu

namespace {

constexpr size_t kNoAllocBytes = 32u << 20;
constexpr int kNoAllocSpill = 1024;   // traversal spill entries per warp
constexpr int kNoAllocMaxWarps = 2560;
constexpr int kNoAllocPend = 1 << 16;  // triangle pairs left to the FP64 re-test

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct Layout {
  size_t counters, hist, round_off, meta, perm, pend, warps, end;
  size_t per_warp_entries;
};

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

Layout layout()
{
  Layout L;
  size_t o = 0;
  L.counters = o; o = align256(o + 64 * sizeof(unsigned int));
  L.hist = o; o = align256(o + (kgpu::kMaxSteps + 2) * sizeof(int));
  L.round_off = o; o = align256(o + (kgpu::kMaxSteps + 2) * sizeof(int));
  L.meta = o; o = align256(o + (4 + 2 * (kgpu::kMaxSteps + 2)) * sizeof(int));
  L.perm = o; o = align256(o + (size_t)KGPU_NOALLOC_MAX_EDGES * sizeof(int));
  L.pend = o; o = align256(o + (size_t)kNoAllocPend * sizeof(uint4));
  L.per_warp_entries = (size_t)kgpu::engine_scratch_doubles() + kNoAllocSpill;  // uint2 entries
  L.warps = o; o = align256(o + (size_t)kNoAllocMaxWarps * L.per_warp_entries * sizeof(uint2));
  L.end = o;
  return L;
}

std::mutex g_mu;
void* g_addr[256] = {};  // per device

// the array's device address on the current device, looked up once
cudaError_t scratch_address(unsigned char** base)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    if ((e = cudaGetSymbolAddress(&p, g_noalloc_scratch)) != cudaSuccess) return e;
    if (!p) return cudaErrorInvalidSymbol;
    g_addr[dev] = p;
  }
  *base = (unsigned char*)g_addr[dev];
  return cudaSuccess;
}

}  // namespace

namespace kgpu {
// Called by kgpu_world_create on the world's device: loads the array and
// caches its address, so that kgpu_check_edges_noalloc allocates nothing.
cudaError_t noalloc_prepare()
{
  unsigned char* base = nullptr;
  return scratch_address(&base);
}
}  // namespace kgpu

extern "C" kgpu_status kgpu_check_edges_noalloc(kgpu_world w, int32_t robot, const float* qa, const float* qb,
                                                const int32_t* nsteps, int32_t E, int32_t* first_hit,
                                                kgpu_stream stream);

extern "C" kgpu_status kgpu_check_edges_noalloc(kgpu_world w, int32_t robot, const float* qa, const float* qb,
                                                const int32_t* nsteps, int32_t E, int32_t* first_hit,
                                                kgpu_stream stream)
{
  using kgpu::record_error;
  if (!w || robot < 0 || robot >= (int)w->robots.size())
    return record_error(KGPU_ERR_INVALID, "kgpu_check_edges_noalloc: null world or robot index out of range");
  if (E < 0 || E > KGPU_NOALLOC_MAX_EDGES)
    return record_error(KGPU_ERR_INVALID,
                        "kgpu_check_edges_noalloc: E must be in [0, 65536] (the fixed scratch holds at most "
                        "KGPU_NOALLOC_MAX_EDGES edges); split the batch or use kgpu_check_edges");
  if (E > 0 && (!qa || !qb || !nsteps || !first_hit))
    return record_error(KGPU_ERR_INVALID, "kgpu_check_edges_noalloc: null buffer");
  if (w->tables_dirty)
    return record_error(KGPU_ERR_INVALID,
                        "kgpu_check_edges_noalloc: collision masks changed since the last query; re-uploading "
                        "them allocates, so run one regular query (e.g. kgpu_check_edges) first");
  if (E == 0) return KGPU_OK;
  const Layout L = layout();
  if (L.end > kNoAllocBytes)
    return record_error(KGPU_ERR_UNSUPPORTED, "kgpu_check_edges_noalloc: scratch layout exceeds the static array");
  const int warps = kgpu::engine_warps_per_block();
  // the main pass runs per_sm blocks per SM; its FP64 fallback pass runs two
  // per SM: both must fit the per-warp regions
  if (2 * w->num_sms * warps > kNoAllocMaxWarps)
    return record_error(KGPU_ERR_UNSUPPORTED,
                        "kgpu_check_edges_noalloc: the static scratch serves GPUs of at most 160 SMs");
  unsigned char* base = nullptr;
  if (scratch_address(&base) != cudaSuccess)
    return record_error(KGPU_ERR_CUDA, "kgpu_check_edges_noalloc: cudaGetSymbolAddress of the scratch failed");
  kgpu::Scratch S;
  S.counters = (unsigned int*)(base + L.counters);
  S.edge_hist = (int*)(base + L.hist);
  S.edge_round_off = (int*)(base + L.round_off);
  S.edge_meta = (int*)(base + L.meta);
  S.edge_perm = (int*)(base + L.perm);
  S.pend = (uint4*)(base + L.pend);
  S.pend_cap = kNoAllocPend;
  S.edge_cap = KGPU_NOALLOC_MAX_EDGES;
  S.spill = (uint2*)(base + L.warps);
  S.spill_per_warp = L.per_warp_entries;
  S.max_warps = kNoAllocMaxWarps;
  S = kgpu::engine_scratch(w, S);  // the world's caps, if any, below the array's sizes
  // the world's tuned launch shape, with as many blocks per SM as the
  // per-warp regions serve
  int per_sm = w->blocks_per_sm;
  while (per_sm > 1 && w->num_sms * per_sm * warps > kNoAllocMaxWarps) --per_sm;
  cudaError_t e = kgpu::launch_check_edges(w->d_dev, w->d_status, S, robot, qa, qb, nsteps, E, first_hit,
                                           w->num_sms * per_sm, per_sm, (cudaStream_t)stream, w->grab, w->job_flush,
                                           w->edge_chunk, w->fp64_inline);
  if (e != cudaSuccess) return record_error(KGPU_ERR_CUDA, cudaGetErrorString(e));
  return KGPU_OK;
}
