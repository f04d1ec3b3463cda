// femtc_batch_apply_static: the batched launch for callers that cannot
// allocate device memory.
//
// femtc_batch_create keeps its tile schedule and mesh table in device memory
// it allocates with cudaMalloc.  Some callers cannot allow that: code that
// runs while another thread captures a CUDA graph in global capture mode
// (cudaMalloc is then an error), applications whose memory manager has
// reserved the device's memory up front, and latency-bound loops that must
// not take cudaMalloc's implicit device synchronisation.  This entry point
// runs the same batch kernel with the schedule and the mesh table placed in
// a fixed array in this file (g_batch_scratch, kStaticScratchBytes), which
// every GPU that loads the library holds until the process exits.
//
// * The first call on a device looks up the array's device address with
//   cudaGetSymbolAddress (with that device current); make that first call
//   before any stream capture.
// * Every call reuses the array.  Nothing in it must start at zero: each
//   call writes the whole mesh table and tile schedule it reads.  Calls on
//   one stream are ordered; calls whose work overlaps on the GPU (other
//   streams, other host threads) race on the array.
// * A batch whose schedule does not fit is rejected with FEMTC_ERR_INVALID
//   and a message giving the capacity.
// * No cudaMalloc, cudaFree or other allocating routine is called: the
//   schedule is uploaded with cudaMemcpyAsync on the caller's stream, from
//   host vectors that are freed when the call returns.  A copy recorded into
//   a CUDA graph would keep pointers to that freed memory, so the call
//   returns FEMTC_ERR_UNSUPPORTED, before any work, when `stream` is
//   capturing.
#include "batch_host.hpp"

#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

namespace femtc
{
int aux_fail(int code, const char* msg); // femtc_abi.cu

namespace
{
// The mesh table (kStaticMaxItems entries at most) followed by the tile
// schedule of one call.
constexpr size_t kStaticScratchBytes = size_t(8) << 20; // 8 MiB
constexpr int kStaticMaxItems = 4096;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_batch_scratch[kStaticScratchBytes];

std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_batch_scratch on the current device (set up once per
// device, with that device current).
int scratch_address(void** out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return aux_fail(FEMTC_ERR_UNSUPPORTED, "batch_apply_static: device index above 63");
  std::lock_guard<std::mutex> lk(g_scratch_mutex);
  if (!g_scratch_addr[dev])
  {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_batch_scratch);
    if (e != cudaSuccess || !p)
      return aux_fail(FEMTC_ERR_CUDA, "batch_apply_static: cudaGetSymbolAddress failed");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return FEMTC_OK;
}

size_t round256(size_t x) { return (x + 255) & ~size_t(255); }
} // namespace
} // namespace femtc

using namespace femtc;

extern "C" int femtc_batch_apply_static(int dtype, const femtc_batch_item* items,
                                        int nitems, void* stream)
{
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t ce = cudaStreamIsCapturing(st, &cs);
  if (ce != cudaSuccess)
  {
    cudaGetLastError();
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(ce));
  }
  if (cs != cudaStreamCaptureStatusNone)
    return aux_fail(FEMTC_ERR_UNSUPPORTED,
                    "batch_apply_static: the stream is capturing; the schedule upload reads "
                    "host memory that the call frees on return");
  if (nitems > kStaticMaxItems)
  {
    char msg[160];
    std::snprintf(msg, sizeof(msg),
                  "batch_apply_static: %d meshes exceed the static capacity of %d meshes",
                  nitems, kStaticMaxItems);
    return aux_fail(FEMTC_ERR_INVALID, msg);
  }
  // the batch's host description; it owns no device memory
  femtc_batch b;
  int rc = batch_setup(&b, dtype, items, nitems, "batch_apply_static");
  if (rc != FEMTC_OK)
    return rc;
  const BatchKernelInfo* fam = b.fam;
  b.threads = batch_default_threads(*fam);
  const std::vector<BatchLayout> lay = batch_default_layouts(*fam, b.threads, b.items);
  std::vector<BatchTile> order;
  rc = batch_plan(&b, lay, order);
  if (rc != FEMTC_OK)
    return rc;
  std::vector<BatchItem<float>> table;
  batch_item_table(&b, table);
  const size_t items_bytes = round256(sizeof(BatchItem<float>) * table.size());
  const size_t tiles_bytes = sizeof(BatchTile) * order.size();
  if (items_bytes + tiles_bytes > kStaticScratchBytes)
  {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "batch_apply_static: %zu tiles exceed the static capacity of %zu tiles "
                  "(%zu bytes)",
                  order.size(), (kStaticScratchBytes - items_bytes) / sizeof(BatchTile),
                  kStaticScratchBytes);
    return aux_fail(FEMTC_ERR_INVALID, msg);
  }
  void* base = nullptr;
  rc = scratch_address(&base);
  if (rc != FEMTC_OK)
    return rc;
  unsigned char* p = static_cast<unsigned char*>(base);
  cudaError_t e = cudaMemcpyAsync(p, table.data(), sizeof(BatchItem<float>) * table.size(),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(p + items_bytes, order.data(), tiles_bytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  b.params.items = reinterpret_cast<const BatchItem<float>*>(p);
  b.params.tiles = reinterpret_cast<const BatchTile*>(p + items_bytes);
  void* args[] = {&b.params};
  e = cudaLaunchKernel(fam->fn, dim3((unsigned)b.grid), dim3((unsigned)b.threads), args, b.smem,
                       st);
  if (e != cudaSuccess)
    return aux_fail(FEMTC_ERR_CUDA, cudaGetErrorString(e));
  return FEMTC_OK;
}
