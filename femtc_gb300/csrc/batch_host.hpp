// Host-side state of a batched launch, shared by the translation units that
// build and launch batches (batch.cu and friends).
#pragma once

#include "femtc_gpu.h"

#include "batch_kernel.cuh"

#include <memory>
#include <vector>

struct femtc_batch
{
  // A mesh run by the library's single-mesh operator kernels inside the
  // batch's graph (split plan), with its own copy of the tables.
  struct Solo
  {
    femtc_batch_item it;
    std::vector<float> tab;
  };

  int dtype = 0;
  const femtc::BatchKernelInfo* fam = nullptr;
  std::vector<femtc_batch_item> items;
  femtc::BatchParams<float> params;
  femtc::BatchTile* d_tiles = nullptr;
  femtc::BatchItem<float>* d_items = nullptr;
  long long ntiles = 0;
  int grid = 0;
  int threads = femtc::kCellThreads; // per CTA (the tile code is blockDim-generic)
  unsigned min_smem = 0;             // shared memory at least (tuner sub-batches)
  unsigned smem = 0;
  long long ndofs = 0;
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // Split plan: the graph's parallel branches (streams and the fork and
  // join events of the capture)
  static constexpr int kBranches = 4;
  cudaStream_t side[kBranches] = {};
  cudaEvent_t fork_ev = nullptr;
  cudaEvent_t join_ev[kBranches] = {};
  // Split plan (chosen by the tuner when faster than one kernel over the
  // whole mix): one batch kernel per variant whose meshes run best
  // persistent, and single-mesh launches for the variants whose meshes are
  // large enough to run best alone.  Empty: the one-kernel plan above.
  std::vector<std::unique_ptr<femtc_batch>> parts;
  std::vector<Solo> solo;

  ~femtc_batch()
  {
    if (exec)
      cudaGraphExecDestroy(exec);
    if (graph)
      cudaGraphDestroy(graph);
    if (cap_stream)
      cudaStreamDestroy(cap_stream);
    for (int k = 0; k < kBranches; ++k)
    {
      if (side[k])
        cudaStreamDestroy(side[k]);
      if (join_ev[k])
        cudaEventDestroy(join_ev[k]);
    }
    if (fork_ev)
      cudaEventDestroy(fork_ev);
    if (d_tiles)
      cudaFree(d_tiles);
    if (d_items)
      cudaFree(d_items);
  }
};

namespace femtc
{
// Kernel family of a batch dtype (FEMTC_F32, FEMTC_F16X2, FEMTC_BF16X3).
const BatchKernelInfo* batch_family_for(int dtype);
// Validate the meshes of a batch and fill b's items and per-degree tables;
// FP32 batches whose tables are all symmetric take the even-odd family.
// `who` prefixes the error messages.
int batch_setup(femtc_batch* b, int dtype, const femtc_batch_item* items, int nitems,
                const char* who);
// Built-in tile layouts (one per variant) of the batch kernel with `threads`
// threads per CTA for a mix of meshes: within the shared memory that keeps
// the CTAs per SM its registers allow.
std::vector<BatchLayout> batch_default_layouts(const BatchKernelInfo& fam, int threads,
                                               const std::vector<femtc_batch_item>& items);
// Built-in threads per CTA of a family's batch kernel.
int batch_default_threads(const BatchKernelInfo& fam);
// Host plan of a batch: stage sizes, shared memory, grid and tile order.
int batch_plan(femtc_batch* b, const std::vector<BatchLayout>& lay,
               std::vector<BatchTile>& order);
// Device mesh table of a batch (pointers of its items).
void batch_item_table(const femtc_batch* b, std::vector<BatchItem<float>>& items);
} // namespace femtc
