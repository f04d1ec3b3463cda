// Host side of the batched persistent launch (femtc_batch_* in femtc_gpu.h):
// validation, per-degree table slots, per-variant tile layouts (built-in or
// measured by the autotuner), the longest-processing-time static schedule,
// device descriptor tables, and the CUDA-graph capture of the launch.
#include "femtc_gpu.h"

#include "batch_host.hpp"
#include "registry.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <queue>
#include <vector>

namespace femtc
{
int aux_fail(int code, const char* msg); // femtc_abi.cu
std::pair<int, int> slab_layout_for(int n, int q, int esize, int lanes); // femtc_abi.cu

namespace
{
constexpr unsigned kBatchSmemCap = 220u * 1024u;

// Shared memory one CTA of the batch kernel may take without lowering the
// number of CTAs per SM that its registers allow (the kernel's register
// count is its largest variant's, so registers set the occupancy and shared
// memory is sized to it).
unsigned smem_budget(const BatchKernelInfo& fam, int threads)
{
  cudaFuncAttributes a{};
  int dev = 0, regs_sm = 65536, smem_sm = 228 * 1024;
  if (cudaFuncGetAttributes(&a, fam.fn) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess)
    return 104u * 1024u;
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  const int warps = (threads + 31) / 32;
  const int regs_warp = (a.numRegs * 32 + 255) / 256 * 256; // allocation unit: 256
  const int ctas = std::max(1, std::min(8, regs_sm / std::max(1, regs_warp * warps)));
  const long long b = (long long)smem_sm / ctas - 1024 - (long long)a.sharedSizeBytes;
  return (unsigned)std::max<long long>(16 * 1024, std::min<long long>(b, kBatchSmemCap));
}

// Variants present in a list of meshes.
std::vector<char> variants_present(const std::vector<femtc_batch_item>& items)
{
  std::vector<char> present(kBatchVariants, 0);
  for (const femtc_batch_item& it : items)
    present[batch_variant(it.op, it.degree + 1)] = 1;
  return present;
}

// Shared memory of a batch CTA: the stages hold the largest tile of the
// variants present (3 x DOF/output stage, 2 x geometry stage, work).
unsigned smem_of_mix(const BatchKernelInfo& fam, const std::vector<char>& present,
                     const std::vector<BatchLayout>& lay, unsigned* su_out = nullptr,
                     unsigned* sg_out = nullptr, unsigned* sw_out = nullptr)
{
  unsigned su = 0, sg = 0, sw = 0;
  for (int v = 0; v < kBatchVariants; ++v)
    if (present[v])
    {
      unsigned bu, bg, bw;
      fam.bytes(v, lay[v], &bu, &bg, &bw);
      su = std::max(su, (bu + 15u) & ~15u);
      sg = std::max(sg, (bg + 15u) & ~15u);
      sw = std::max(sw, (bw + 15u) & ~15u);
    }
  if (su_out)
    *su_out = su;
  if (sg_out)
    *sg_out = sg;
  if (sw_out)
    *sw_out = sw;
  return 128 + 2 * (su + sg) + su + sw;
}

const BatchKernelInfo* family_for(int dtype)
{
  static const BatchKernelInfo f32 = batch_kernel_f32();
  static const BatchKernelInfo f16 = batch_kernel_f16x2();
  static const BatchKernelInfo bf16 = batch_kernel_bf16x3();
  switch (dtype)
  {
  case FEMTC_F32: return &f32;
  case FEMTC_F16X2: return &f16;
  case FEMTC_BF16X3: return &bf16;
  default: return nullptr;
  }
}

double cell_cost(int op, int n)
{
  // bytes + flops/8 per cell (FP32 storage): the schedule's cost model
  const double q = n + 1;
  const double bytes = 4.0 * (2.0 * n * n * n + (op ? 6.0 : 1.0) * q * q * q);
  const double flops = op ? 4.0 * q * n * (2.0 * n * n + 3.0 * q * n + 3.0 * q * q) + 15.0 * q * q * q
                          : 4.0 * q * n * (n * n + q * n + q * q) + q * q * q;
  return bytes + flops / 8.0;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
} // namespace
} // namespace femtc

using namespace femtc;


namespace femtc
{
namespace
{
} // namespace

const BatchKernelInfo* batch_family_for(int dtype) { return family_for(dtype); }

void register_batch_faults(std::vector<FaultReader>& f)
{
  f.push_back(batch_kernel_f32().read_fault);
  f.push_back(batch_kernel_f32eo().read_fault);
  f.push_back(batch_kernel_f16x2().read_fault);
  f.push_back(batch_kernel_bf16x3().read_fault);
}

bool even_odd_tables_f32(const float* tab, int n, int q, int ntab); // femtc_abi.cu

int batch_setup(femtc_batch* b, int dtype, const femtc_batch_item* items, int nitems,
                const char* who)
{
  char msg[160];
  auto bad = [&](int code, const char* what) -> int {
    std::snprintf(msg, sizeof(msg), "%s: %s", who, what);
    return aux_fail(code, msg);
  };
  const BatchKernelInfo* fam = family_for(dtype);
  if (!fam)
    return bad(FEMTC_ERR_UNSUPPORTED, "dtype must be FEMTC_F32, FEMTC_F16X2 or FEMTC_BF16X3");
  if (!items || nitems < 1)
    return bad(FEMTC_ERR_INVALID, "no items");
  b->dtype = dtype;
  b->fam = fam;
  std::memset(&b->params, 0, sizeof(b->params));
  char slot_set[kBatchDegrees] = {};
  for (int i = 0; i < nitems; ++i)
  {
    const femtc_batch_item& it = items[i];
    if (it.op != FEMTC_OP_MASS && it.op != FEMTC_OP_STIFFNESS)
      return bad(FEMTC_ERR_INVALID, "bad op");
    if (it.degree < 1 || it.degree > kBatchDegrees)
      return bad(FEMTC_ERR_UNSUPPORTED, "degree must be in 1..7");
    if (it.nquad != it.degree + 2)
      return bad(FEMTC_ERR_UNSUPPORTED, "nquad must be degree+2");
    if (!it.tables || !it.u || !it.y || !it.geo)
      return bad(FEMTC_ERR_INVALID, "null pointer in an item");
    if (!aligned16(it.u) || !aligned16(it.y) || !aligned16(it.geo))
      return bad(FEMTC_ERR_INVALID, "device pointers must be 16-byte aligned");
    const int n = it.degree + 1, q = it.nquad, slot = n - 2;
    const int ntab = it.op == FEMTC_OP_STIFFNESS ? 2 : 1;
    const float* t = static_cast<const float*>(it.tables);
    for (int w = 0; w < ntab; ++w)
    {
      float* dst = b->params.tabs[slot][w];
      if (slot_set[slot] & (1 << w))
      {
        if (std::memcmp(dst, t + w * q * n, sizeof(float) * q * n) != 0)
          return bad(FEMTC_ERR_INVALID, "meshes of the same degree must share their tables");
      }
      else
      {
        std::memcpy(dst, t + w * q * n, sizeof(float) * q * n);
        slot_set[slot] |= (char)(1 << w);
      }
    }
    b->items.push_back(it);
    b->ndofs += (long long)it.ncells * n * n * n;
  }
  // FP32 with symmetric tables everywhere: the even-odd family, whose
  // per-degree tables are the even-odd forms of Phi, Gamma, Phi^T, Gamma^T
  if (dtype == FEMTC_F32)
  {
    bool eo = true;
    for (int slot = 0; slot < kBatchDegrees && eo; ++slot)
      if (slot_set[slot])
      {
        const int n = slot + 2, q = n + 1;
        float both[2 * kMaxQ * kMaxN];
        std::memcpy(both, b->params.tabs[slot][0], sizeof(float) * q * n);
        std::memcpy(both + q * n, b->params.tabs[slot][1], sizeof(float) * q * n);
        eo = even_odd_tables_f32(both, n, q, (slot_set[slot] & 2) ? 2 : 1);
      }
    if (eo)
    {
      static const BatchKernelInfo f32eo = batch_kernel_f32eo();
      b->fam = &f32eo;
      for (int slot = 0; slot < kBatchDegrees; ++slot)
        if (slot_set[slot])
        {
          const int n = slot + 2, q = n + 1;
          float plain[2][kMaxQ * kMaxN];
          std::memcpy(plain, b->params.tabs[slot], sizeof(plain));
          for (int w = 0; w < 2; ++w)
          {
            const int sig = w == 0 ? 1 : -1;
            host_eo_table<float>(plain[w], q, n, 1, q, sig, b->params.tabs[slot][w]);
            host_eo_table<float>(plain[w], n, q, q, 1, sig, b->params.tabs[slot][2 + w]);
          }
        }
    }
  }
  return FEMTC_OK;
}

namespace
{
// Default layout of a variant for the batch kernel with `threads` threads
// per CTA: the best lane efficiency for tiles whose own stages fit `budget`.
BatchLayout default_batch_layout(const BatchKernelInfo& fam, int v, int threads, unsigned budget)
{
  const int op = v / kBatchDegrees, n = 2 + v % kBatchDegrees, q = n + 1;
  const int lanes = fam.family == kFamilySlab
                        ? batch_slab_lanes(op == 0 ? OP_MASS : OP_STIFFNESS, n)
                        : 1; // even-odd and tensor-core tiles: one lane
  BatchLayout best{4, 0, 0, 0};
  if (slab_family(fam.family))
  {
    auto l = slab_layout_for(n, q, 4, lanes);
    best.sq = l.first;
    best.sbc = l.second;
  }
  double best_score = -1.0;
  for (int cb = 4; cb <= 128; cb += 4)
  {
    BatchLayout l = best;
    l.cb = cb;
    l.staged = 0;
    unsigned bu, bg, bw;
    fam.bytes(v, l, &bu, &bg, &bw);
    if (128 + 3 * bu + 2 * bg + bw > budget)
      break;
    // busy lanes of the slab passes and of the pencil pass: per warp (its
    // block of cells) for the CUDA-core families, per CTA for tensor cores
    const bool split = slab_family(fam.family);
    const double cells = split ? std::ceil((double)cb / (threads / 32)) : cb;
    const int width = split ? 32 : threads;
    const double busy[2] = {cells * n * lanes, cells * q * q};
    double eff = 0.0;
    for (double x : busy)
      eff += x / (std::ceil(x / width) * width);
    const double score = eff + 1e-4 * cb;
    if (score > best_score)
    {
      best_score = score;
      best = l;
    }
  }
  return best;
}

// Default layouts of a mix: every variant's own best, then the tiles that
// set the stage maxima shrink (4 cells at a time) until the mix fits the
// budget.
std::vector<BatchLayout> default_batch_layouts(const BatchKernelInfo& fam, int threads,
                                               const std::vector<char>& present)
{
  const unsigned budget = smem_budget(fam, threads);
  std::vector<BatchLayout> lay(kBatchVariants);
  for (int v = 0; v < kBatchVariants; ++v)
    lay[v] = default_batch_layout(fam, v, threads, budget);
  unsigned total = smem_of_mix(fam, present, lay);
  while (total > budget)
  {
    int best_v = -1;
    unsigned best_total = total;
    for (int v = 0; v < kBatchVariants; ++v)
    {
      if (!present[v] || lay[v].cb <= 4)
        continue;
      std::vector<BatchLayout> trial = lay;
      trial[v].cb -= 4;
      const unsigned t = smem_of_mix(fam, present, trial);
      if (t < best_total)
      {
        best_total = t;
        best_v = v;
      }
    }
    if (best_v < 0)
      break; // every tile at its minimum: the plan runs with fewer CTAs per SM
    lay[best_v].cb -= 4;
    total = best_total;
  }
  return lay;
}

// Threads per CTA without tuning.  The plain CUDA-core family needs about
// 255 registers per thread (the whole slab of a degree-7 cell), so a
// 256-thread CTA is alone on its SM and every barrier of a tile idles the
// SM; two 128-thread CTAs per SM overlap one another's barriers and TMA
// waits.  The even-odd and tensor-core families fit in 128 registers and
// run two 256-thread CTAs per SM.
int default_threads(const BatchKernelInfo& fam)
{
  return fam.family == kFamilySlab ? 128 : kCellThreads;
}

} // namespace

// Host part of a batch build: stage sizes, shared memory, grid, and the
// longest-processing-time tile order (CTA g runs order[g], order[g+G], ...).
// No device memory is allocated here.
int batch_plan(femtc_batch* b, const std::vector<BatchLayout>& lay,
               std::vector<BatchTile>& order)
{
  const BatchKernelInfo& fam = *b->fam;
  BatchParams<float>& p = b->params;
  for (int v = 0; v < kBatchVariants; ++v)
    p.lay[v] = lay[v];
  // stage sizes: max over the variants present (work buffers at least as
  // large as the batch's min_smem asks, so that a sub-batch timed by the
  // tuner runs at the full batch's occupancy)
  unsigned su = 0, sg = 0, sw = 0;
  const unsigned mix = smem_of_mix(fam, variants_present(b->items), lay, &su, &sg, &sw);
  if (b->min_smem > mix)
    sw += (b->min_smem - mix + 15u) & ~15u;
  p.stage_u = su;
  p.stage_g = sg;
  p.stage_y = su;
  b->smem = 128 + 2 * (su + sg) + su + sw;
  if (b->smem > kBatchSmemCap)
    return aux_fail(FEMTC_ERR_INVALID, "batch: tile stages exceed shared memory");
  {
    // the kernel's shared-memory limit only grows: batches (and the parts of
    // a split batch) built earlier keep launching with their own sizes
    static std::mutex m;
    static std::map<const void*, unsigned> limit;
    std::lock_guard<std::mutex> lk(m);
    unsigned& cur = limit[fam.fn];
    if (b->smem > cur)
    {
      cudaError_t e = cudaFuncSetAttribute(fam.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)b->smem);
      if (e != cudaSuccess)
        return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
      cur = b->smem;
    }
  }
  int per_sm = 0, dev = 0, sms = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fam.fn, b->threads, b->smem);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (per_sm < 1)
    return aux_fail(FEMTC_ERR_UNSUPPORTED, "batch kernel does not fit on an SM");

  // tiles and their costs
  struct Work
  {
    BatchTile t;
    double cost;
  };
  std::vector<Work> work;
  for (size_t i = 0; i < b->items.size(); ++i)
  {
    const femtc_batch_item& it = b->items[i];
    const int v = batch_variant(it.op, it.degree + 1);
    const int cb = lay[v].cb;
    const double c = cell_cost(it.op, it.degree + 1);
    for (long long c0 = 0; c0 < (long long)it.ncells; c0 += cb)
    {
      const int ncb = (int)std::min<long long>(cb, (long long)it.ncells - c0);
      work.push_back({BatchTile{c0, (int)i, v, ncb, ncb == cb ? 1 : 0}, c * ncb});
    }
  }
  const long long nwork = (long long)work.size();
  b->grid = (int)std::max<long long>(1, std::min<long long>(nwork, (long long)per_sm * sms));
  // longest processing time first onto the least loaded CTA
  std::stable_sort(work.begin(), work.end(),
                   [](const Work& a, const Work& c) { return a.cost > c.cost; });
  using Slot = std::pair<double, int>;
  std::priority_queue<Slot, std::vector<Slot>, std::greater<Slot>> heap;
  for (int g = 0; g < b->grid; ++g)
    heap.push({0.0, g});
  std::vector<std::vector<BatchTile>> per(b->grid);
  for (const Work& w : work)
  {
    Slot s = heap.top();
    heap.pop();
    per[s.second].push_back(w.t);
    heap.push({s.first + w.cost, s.second});
  }
  size_t rounds = 0;
  for (auto& v : per)
    rounds = std::max(rounds, v.size());
  order.assign(rounds * b->grid, BatchTile{0, -1, 0, 0, 0});
  for (int g = 0; g < b->grid; ++g)
    for (size_t j = 0; j < per[g].size(); ++j)
      order[j * b->grid + g] = per[g][j];
  b->ntiles = (long long)order.size();
  p.ntiles = b->ntiles;
  return FEMTC_OK;
}

// Device mesh table of a batch.
void batch_item_table(const femtc_batch* b, std::vector<BatchItem<float>>& items)
{
  items.resize(b->items.size());
  for (size_t i = 0; i < b->items.size(); ++i)
    items[i] = BatchItem<float>{static_cast<const float*>(b->items[i].u),
                                static_cast<float*>(b->items[i].y),
                                static_cast<const float*>(b->items[i].geo)};
}

namespace
{
} // namespace

std::vector<BatchLayout> batch_default_layouts(const BatchKernelInfo& fam, int threads,
                                               const std::vector<femtc_batch_item>& items)
{
  return default_batch_layouts(fam, threads, variants_present(items));
}

int batch_default_threads(const BatchKernelInfo& fam) { return default_threads(fam); }

namespace
{
int build(femtc_batch* b, const std::vector<BatchLayout>& lay)
{
  std::vector<BatchTile> order;
  int rc = batch_plan(b, lay, order);
  if (rc != FEMTC_OK)
    return rc;
  BatchParams<float>& p = b->params;
  std::vector<BatchItem<float>> items;
  batch_item_table(b, items);
  if (b->d_tiles)
    cudaFree(b->d_tiles);
  if (b->d_items)
    cudaFree(b->d_items);
  b->d_tiles = nullptr;
  b->d_items = nullptr;
  if (cudaMalloc(&b->d_tiles, sizeof(BatchTile) * std::max<size_t>(1, order.size())) !=
          cudaSuccess ||
      cudaMalloc(&b->d_items, sizeof(BatchItem<float>) * std::max<size_t>(1, items.size())) !=
          cudaSuccess)
    return aux_fail(FEMTC_ERR_NOMEM, "batch: descriptor allocation failed");
  cudaMemcpy(b->d_tiles, order.data(), sizeof(BatchTile) * order.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_items, items.data(), sizeof(BatchItem<float>) * items.size(),
             cudaMemcpyHostToDevice);
  p.tiles = b->d_tiles;
  p.items = b->d_items;
  return FEMTC_OK;
}

int launch_solo(int dtype, const femtc_batch::Solo& s, cudaStream_t st)
{
  const femtc_batch_item& it = s.it;
  return it.op == FEMTC_OP_MASS
             ? femtc_mass_apply(dtype, FEMTC_EXACT, it.degree, it.nquad, s.tab.data(), it.u,
                                it.y, it.geo, it.ncells, st)
             : femtc_stiffness_apply(dtype, FEMTC_EXACT, it.degree, it.nquad, s.tab.data(),
                                     it.u, it.y, it.geo, it.ncells, st);
}

int launch_eager(femtc_batch* b, cudaStream_t st)
{
  if (!b->parts.empty() || !b->solo.empty())
  {
    for (auto& p : b->parts)
    {
      const int rc = launch_eager(p.get(), st);
      if (rc != FEMTC_OK)
        return rc;
    }
    for (const auto& s : b->solo)
    {
      const int rc = launch_solo(b->dtype, s, st);
      if (rc != FEMTC_OK)
        return rc;
    }
    return FEMTC_OK;
  }
  void* args[] = {&b->params};
  cudaError_t e = cudaLaunchKernel(b->fam->fn, dim3((unsigned)b->grid), dim3((unsigned)b->threads),
                                   args, b->smem, st);
  return e == cudaSuccess ? FEMTC_OK : aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
}

// Split plan: the batch kernels and single-mesh launches write disjoint
// outputs, so the graph runs them on parallel branches, each launch on the
// branch with the least estimated work so far (longest first): small
// launches overlap one another and the tails of the large ones instead of
// running one after another on a mostly idle GPU.
int capture_branches(femtc_batch* b)
{
  constexpr int K = femtc_batch::kBranches;
  for (int k = 0; k < K; ++k)
  {
    if (!b->side[k] && cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking) != cudaSuccess)
      return aux_fail(FEMTC_ERR_CUDA, "batch: stream creation failed");
    if (!b->join_ev[k] &&
        cudaEventCreateWithFlags(&b->join_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return aux_fail(FEMTC_ERR_CUDA, "batch: event creation failed");
  }
  if (!b->fork_ev && cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, "batch: event creation failed");
  struct Task
  {
    double cost;
    int part, solo;
  };
  std::vector<Task> tasks;
  for (size_t i = 0; i < b->parts.size(); ++i)
  {
    double c = 0.0;
    for (const auto& it : b->parts[i]->items)
      c += cell_cost(it.op, it.degree + 1) * (double)it.ncells;
    tasks.push_back({c, (int)i, -1});
  }
  for (size_t j = 0; j < b->solo.size(); ++j)
  {
    const femtc_batch_item& it = b->solo[j].it;
    tasks.push_back({cell_cost(it.op, it.degree + 1) * (double)it.ncells, -1, (int)j});
  }
  std::stable_sort(tasks.begin(), tasks.end(),
                   [](const Task& x, const Task& y) { return x.cost > y.cost; });
  cudaEventRecord(b->fork_ev, b->cap_stream);
  for (int k = 0; k < K; ++k)
    cudaStreamWaitEvent(b->side[k], b->fork_ev, 0);
  double load[K] = {};
  int rc = FEMTC_OK;
  for (const Task& t : tasks)
  {
    int k = 0;
    for (int j = 1; j < K; ++j)
      if (load[j] < load[k])
        k = j;
    load[k] += t.cost;
    rc = t.part >= 0 ? launch_eager(b->parts[t.part].get(), b->side[k])
                     : launch_solo(b->dtype, b->solo[t.solo], b->side[k]);
    if (rc != FEMTC_OK)
      break;
  }
  // every branch joins the capture stream, also after an error, so that
  // the capture can end
  for (int k = 0; k < K; ++k)
  {
    cudaEventRecord(b->join_ev[k], b->side[k]);
    cudaStreamWaitEvent(b->cap_stream, b->join_ev[k], 0);
  }
  return rc;
}

int capture(femtc_batch* b)
{
  if (b->exec)
    cudaGraphExecDestroy(b->exec);
  if (b->graph)
    cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  if (!b->cap_stream &&
      cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, "batch: stream creation failed");
  cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  int rc = (!b->parts.empty() || !b->solo.empty()) ? capture_branches(b)
                                                   : launch_eager(b, b->cap_stream);
  e = cudaStreamEndCapture(b->cap_stream, &b->graph);
  if (rc != FEMTC_OK)
    return rc;
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  return e == cudaSuccess ? FEMTC_OK : aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
}

float time_launches(femtc_batch* b, cudaStream_t st, int reps)
{
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch_eager(b, st);
  cudaEventRecord(e0, st);
  for (int r = 0; r < reps; ++r)
    launch_eager(b, st);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

// Autotuner of the batch: for every variant present, time candidate tile
// shapes on that variant's meshes alone (the batch kernel, same stage
// budget) and keep the fastest.
void tune_layouts(femtc_batch* b, std::vector<BatchLayout>& lay, cudaStream_t st)
{
  const std::vector<femtc_batch_item> all = b->items;
  const std::vector<char> present = variants_present(all);
  const unsigned budget = smem_budget(*b->fam, b->threads);
  for (int v = 0; v < kBatchVariants; ++v)
  {
    std::vector<femtc_batch_item> mine;
    for (const auto& it : all)
      if (batch_variant(it.op, it.degree + 1) == v)
        mine.push_back(it);
    if (mine.empty())
      continue;
    femtc_batch sub;
    sub.dtype = b->dtype;
    sub.fam = b->fam;
    sub.threads = b->threads;
    sub.items = mine;
    std::memcpy(sub.params.tabs, b->params.tabs, sizeof(b->params.tabs));
    const BatchLayout base = lay[v];
    float best = 1e30f;
    BatchLayout best_l = base;
    for (int staged = 0; staged <= 1; ++staged)
      for (int mult : {1, 2, 3, 4, 6, 8})
      {
        BatchLayout l = base;
        l.cb = std::max(4, (base.cb * mult / 4 + 3) / 4 * 4);
        l.staged = staged;
        std::vector<BatchLayout> trial = lay;
        trial[v] = l;
        // the whole mix must stay within the budget; the sub-batch is timed
        // with the mix's shared memory (same CTAs per SM)
        const unsigned mix = smem_of_mix(*b->fam, present, trial);
        if (mix > budget && !(mult == 1 && staged == 0))
          continue;
        sub.min_smem = mix;
        if (build(&sub, trial) != FEMTC_OK)
          continue;
        const float ms = time_launches(&sub, st, 3);
        if (ms < best)
        {
          best = ms;
          best_l = l;
        }
      }
    lay[v] = best_l;
  }
}

// Threads per CTA and tile layouts: for each candidate CTA size, tune the
// layouts variant by variant, then time the whole batch; keep the fastest.
void tune(femtc_batch* b, std::vector<BatchLayout>& lay)
{
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  float best = 1e30f;
  int best_threads = b->threads;
  std::vector<BatchLayout> best_lay = lay;
  for (int threads : {128, 256})
  {
    b->threads = threads;
    std::vector<BatchLayout> trial =
        default_batch_layouts(*b->fam, threads, variants_present(b->items));
    tune_layouts(b, trial, st);
    if (build(b, trial) != FEMTC_OK)
      continue;
    const float ms = time_launches(b, st, 3);
    if (ms < best)
    {
      best = ms;
      best_threads = threads;
      best_lay = trial;
    }
  }
  b->threads = best_threads;
  lay = best_lay;
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
}

// Mean time (ms) of `reps` runs of `run` on st, after one untimed run.
template <typename F>
float time_runs(F run, cudaStream_t st, int reps)
{
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  run();
  cudaEventRecord(e0, st);
  for (int r = 0; r < reps; ++r)
    run();
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

// Split plan: one kernel over the whole mix sizes its shared memory and
// registers for the largest variant present, so small variants run at the
// occupancy of the largest; and the largest meshes run as fast alone, where
// a launch's overhead is negligible.  For every variant present, time (a)
// a batch of its meshes alone, tuned, and (b) its meshes as single-mesh
// launches with tiles autotuned on the largest; keep the faster of each.
// The split plan replaces the one-kernel plan when the whole of it is
// faster.  The y buffers are overwritten.
void plan_split(femtc_batch* b, bool force)
{
  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
    return;
  const float t_full = time_launches(b, st, 3);
  std::vector<std::unique_ptr<femtc_batch>> parts;
  std::vector<femtc_batch::Solo> solo;
  bool ok = true;
  for (int v = 0; v < kBatchVariants && ok; ++v)
  {
    std::vector<femtc_batch_item> mine;
    for (const auto& it : b->items)
      if (batch_variant(it.op, it.degree + 1) == v)
        mine.push_back(it);
    if (mine.empty())
      continue;
    auto s = std::make_unique<femtc_batch>();
    if (batch_setup(s.get(), b->dtype, mine.data(), (int)mine.size(), "batch") != FEMTC_OK)
    {
      ok = false;
      break;
    }
    s->threads = default_threads(*s->fam);
    std::vector<BatchLayout> lay = batch_default_layouts(*s->fam, s->threads, s->items);
    tune(s.get(), lay);
    if (build(s.get(), lay) != FEMTC_OK)
    {
      ok = false;
      break;
    }
    const float tb = time_launches(s.get(), st, 3);
    std::vector<femtc_batch::Solo> ms;
    size_t big = 0;
    for (size_t i = 0; i < mine.size(); ++i)
    {
      const femtc_batch_item& it = mine[i];
      const size_t ntab = 2 * (size_t)it.nquad * (it.degree + 1);
      const float* t = static_cast<const float*>(it.tables);
      ms.push_back({it, std::vector<float>(t, t + ntab)});
      if (it.ncells > mine[big].ncells)
        big = i;
    }
    float ts = 1e30f;
    int cb = 0, staged = 0, nt = 0;
    float tune_ms = 0.f;
    const femtc_batch_item& bi = mine[big];
    if (femtc_autotune(bi.op, b->dtype, FEMTC_EXACT, bi.degree, bi.nquad, ms[big].tab.data(),
                       bi.u, bi.y, bi.geo, bi.ncells, st, &cb, &staged, &nt, &tune_ms) ==
        FEMTC_OK)
    {
      bool run_ok = true;
      ts = time_runs(
          [&] {
            for (const auto& m : ms)
              run_ok = launch_solo(b->dtype, m, st) == FEMTC_OK && run_ok;
          },
          st, 3);
      if (!run_ok)
        ts = 1e30f;
    }
    if (ts < tb)
      solo.insert(solo.end(), ms.begin(), ms.end());
    else
      parts.push_back(std::move(s));
  }
  if (ok)
  {
    femtc_batch trial;
    trial.dtype = b->dtype;
    trial.parts = std::move(parts);
    trial.solo = std::move(solo);
    const float t_split = time_runs([&] { launch_eager(&trial, st); }, st, 3);
    if (force || t_split < t_full)
    {
      b->parts = std::move(trial.parts);
      b->solo = std::move(trial.solo);
    }
  }
  cudaGetLastError();
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
}
} // namespace
} // namespace femtc

extern "C" {

int femtc_batch_create(int dtype, const femtc_batch_item* items, int nitems,
                       int flags, femtc_batch** out)
{
  if (!out)
    return aux_fail(FEMTC_ERR_INVALID, "batch: null output");
  *out = nullptr;
  auto b = std::make_unique<femtc_batch>();
  int rc = batch_setup(b.get(), dtype, items, nitems, "batch");
  if (rc != FEMTC_OK)
    return rc;
  const BatchKernelInfo* fam = b->fam;
  b->threads = default_threads(*fam);
  std::vector<BatchLayout> lay = batch_default_layouts(*fam, b->threads, b->items);
  if (flags & FEMTC_BATCH_TUNE)
    tune(b.get(), lay);
  rc = build(b.get(), lay);
  if (rc != FEMTC_OK)
    return rc;
  if (flags & (FEMTC_BATCH_TUNE | FEMTC_BATCH_SPLIT))
    plan_split(b.get(), (flags & FEMTC_BATCH_SPLIT) != 0);
  rc = capture(b.get());
  if (rc != FEMTC_OK)
    return rc;
  *out = b.release();
  return FEMTC_OK;
}

int femtc_batch_launch(femtc_batch* b, void* stream)
{
  if (!b || !b->exec)
    return aux_fail(FEMTC_ERR_INVALID, "batch: not created");
  cudaError_t e = cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? FEMTC_OK : aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
}

int femtc_batch_launch_eager(femtc_batch* b, void* stream)
{
  if (!b)
    return aux_fail(FEMTC_ERR_INVALID, "batch: not created");
  return launch_eager(b, static_cast<cudaStream_t>(stream));
}

int femtc_batch_info(const femtc_batch* b, long long* ntiles, int* ctas,
                     int* smem_bytes, long long* ndofs)
{
  if (!b)
    return aux_fail(FEMTC_ERR_INVALID, "batch: not created");
  long long nt = b->ntiles;
  int grid = b->grid;
  unsigned smem = b->smem;
  if (!b->parts.empty() || !b->solo.empty())
  {
    // split plan: tiles of the batch kernels plus one per single-mesh launch
    nt = (long long)b->solo.size();
    grid = 0;
    smem = 0;
    for (const auto& p : b->parts)
    {
      nt += p->ntiles;
      grid = std::max(grid, p->grid);
      smem = std::max(smem, p->smem);
    }
  }
  if (ntiles)
    *ntiles = nt;
  if (ctas)
    *ctas = grid;
  if (smem_bytes)
    *smem_bytes = (int)smem;
  if (ndofs)
    *ndofs = b->ndofs;
  return FEMTC_OK;
}

int femtc_batch_plan(const femtc_batch* b, int* kernels, int* single_launches)
{
  if (!b)
    return aux_fail(FEMTC_ERR_INVALID, "batch: not created");
  const bool split = !b->parts.empty() || !b->solo.empty();
  if (kernels)
    *kernels = split ? (int)b->parts.size() : 1;
  if (single_launches)
    *single_launches = (int)b->solo.size();
  return FEMTC_OK;
}

int femtc_batch_layout(const femtc_batch* b, int op, int degree, int* cb,
                       int* geo_staged)
{
  if (!b || degree < 1 || degree > kBatchDegrees || (op != 0 && op != 1))
    return aux_fail(FEMTC_ERR_INVALID, "batch: bad layout query");
  const int v = batch_variant(op, degree + 1);
  const femtc_batch* owner = b;
  if (!b->parts.empty() || !b->solo.empty())
  {
    // split plan: the batch kernel that holds the variant; 0 cells for a
    // variant run by single-mesh launches
    owner = nullptr;
    for (const auto& p : b->parts)
      for (const auto& it : p->items)
        if (batch_variant(it.op, it.degree + 1) == v)
          owner = p.get();
  }
  if (cb)
    *cb = owner ? owner->params.lay[v].cb : 0;
  if (geo_staged)
    *geo_staged = owner ? owner->params.lay[v].staged : 0;
  return FEMTC_OK;
}

int femtc_batch_threads(const femtc_batch* b)
{
  if (!b)
    return aux_fail(FEMTC_ERR_INVALID, "batch: not created");
  if (!b->parts.empty())
  {
    // split plan: the CTA size of the batch kernel with the most tiles
    const femtc_batch* top = b->parts[0].get();
    for (const auto& p : b->parts)
      if (p->ntiles > top->ntiles)
        top = p.get();
    return top->threads;
  }
  return b->solo.empty() ? b->threads : 0;
}

void femtc_batch_destroy(femtc_batch* b) { delete b; }

} // extern "C"
