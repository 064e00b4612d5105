// tree2d_solve_device_static: the device-resident plain solve for callers
// that cannot allocate GPU memory.
//
// Some callers may not call cudaMalloc at all: code that runs inside a host
// application whose GPU memory is owned by a pool it must not bypass, or
// an embedding that forbids allocation after start-up so that its memory
// footprint is fixed.  For them this entry point runs the same kernels as
// tree2d_solve_device, but every scratch buffer (sort buffers, scans,
// cells, coefficients, status word) lives in one file-scope __device__
// array of fixed size, so the call allocates nothing.
//
// Limits and rules (also in include/tree2d.h):
//   - at most kStaticMaxBlobs blobs, and at most the cells that fit in the
//     cell region of the array; larger inputs are rejected with
//     TREE2D_ERR_TOO_LARGE before or during the build;
//   - the array exists once per device and stays resident until the process
//     exits; every call shares it, and it keeps the last call's contents
//     (the solve clears what it reads before writing: the status word and
//     the internal coefficients);
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress); make that first call before any stream capture;
//   - calls that overlap on the GPU race on the array; the call returns only
//     after its work on `stream` is complete, and concurrent host threads are
//     serialised here.
#include <mutex>

#include "dev_common.cuh"

namespace t2d {
namespace {

constexpr int kStaticMaxBlobs = 65536;
constexpr size_t kStaticBytes = size_t(32) << 20;     // 32 MiB per device
constexpr size_t kStatusRegion = 4096;                 // DevStatus
constexpr size_t kBlobRegion = size_t(4) << 20;        // <= 65536 x 48 B
constexpr size_t kTmpRegion = size_t(2) << 20;         // <= 65536 x 20 B + sort counts
constexpr size_t kCellRegion = kStaticBytes - kStatusRegion - kBlobRegion - kTmpRegion;

__device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
unsigned char *g_scratch_ptr[kMaxDevices] = {};
DevStatus g_host_status[2];  // host side of the status readback (pageable)

// Device address of g_static_scratch on the current device.  In host code
// the array's name is only a host-side stand-in; the address must come from
// the runtime, once per device, with that device current.
int scratch_address(unsigned char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    note_cuda_error(e, "cudaGetDevice");
    return TREE2D_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return TREE2D_ERR_NO_DEVICE;
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) {
      note_cuda_error(e, "cudaGetSymbolAddress(g_static_scratch)");
      return TREE2D_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
  }
  *out = g_scratch_ptr[dev];
  return TREE2D_OK;
}

}  // namespace
}  // namespace t2d

using namespace t2d;

extern "C" int tree2d_solve_device_static(int n, const double *d_xy, const double *d_cir, const double *d_cor,
                                          double *d_uv, void *stream) {
  if (n < 0) return record_error(TREE2D_ERR_BAD_INPUT);
  if (n > kStaticMaxBlobs) return record_error(TREE2D_ERR_TOO_LARGE);
  Params p;
  int rc = params_for_device_solve(p);
  if (rc) return rc;
  if (n == 0) return TREE2D_OK;
  std::lock_guard<std::mutex> lk(g_static_mu);
  unsigned char *base = nullptr;
  rc = scratch_address(&base);
  if (rc) return record_error(rc);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  Workspace ws;
  ws.status = reinterpret_cast<DevStatus *>(base);
  ws.h_status = g_host_status;
  ws.blob_arena.attach(base + kStatusRegion, kBlobRegion);
  ws.tmp_arena.attach(base + kStatusRegion + kBlobRegion, kTmpRegion);
  ws.cell_arena.attach(base + kStatusRegion + kBlobRegion + kTmpRegion, kCellRegion);
  ws.init = true;  // nothing else to set up: no events, no pinned memory

  Tree t;
  rc = build_tree(ws, n, d_xy, d_cir, d_cor, p, t, s);
  if (rc == TREE2D_ERR_CUDA && (ws.blob_arena.overflowed() || ws.tmp_arena.overflowed() ||
                                ws.cell_arena.overflowed()))
    rc = TREE2D_ERR_TOO_LARGE;
  if (rc) return record_error(rc);
  rc = plain_upward(ws, t, p, s);
  if (rc) return record_error(rc);
  rc = plain_evaluate(ws, t, p, n, t.x, t.y, t.perm, d_uv, s);
  if (rc) return record_error(rc);
  cudaError_t e = cudaMemcpyAsync(ws.h_status, ws.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    note_cuda_error(e, "tree2d_solve_device_static");
    return record_error(TREE2D_ERR_CUDA);
  }
  if (ws.h_status->err) return record_error(ws.h_status->err);
  return TREE2D_OK;
}
