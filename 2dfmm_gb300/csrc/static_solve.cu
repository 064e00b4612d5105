// tree2d_solve_device_static: the device-resident plain solve for callers
// that cannot allocate GPU memory.
//
// Some callers may not call cudaMalloc at all: code that runs inside a host
// application whose GPU memory is owned by a pool it must not bypass, or
// an embedding that forbids allocation after start-up so that its memory
// footprint is fixed.  For them this entry point runs the same kernels as
// tree2d_solve_device in the plain mode, but every scratch buffer (sort
// buffers, scans, cells, coefficients, status word) lives in one file-scope
// __device__ array of fixed size, so the call allocates nothing.
//
// Limits and rules (also in include/tree2d.h):
//   - plain form only: with the mixed or learned mode in force, or a mirror
//     wall set, the call returns TREE2D_ERR_MODE and computes nothing (it
//     would otherwise answer a different question than tree2d_solve_device);
//   - at most kStaticMaxBlobs blobs, and at most the cells that fit in the
//     cell region of the array; larger inputs are rejected with
//     TREE2D_ERR_TOO_LARGE before or during the build;
//   - the blob and scratch regions are sized, on the first call, from what
//     the tree build itself reserves for kStaticMaxBlobs blobs
//     (build_blob_bytes, build_tmp_bytes), so a buffer added to the build
//     cannot silently push a maximum-size input out of its region;
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
constexpr size_t kStaticBytes = size_t(32) << 20;  // 32 MiB per device
constexpr size_t kStatusRegion = 4096;              // DevStatus
// The blob region holds about 58 B per blob (positions, circulations, core
// radii, 1/sigma^2, permutation, keys, cell bases, two level bytes: 3.8 MB
// at 65,536 blobs), the scratch region about 17 B per blob plus the sort
// counts and the level-12 centre table (1.3 MB); the cells get the rest
// (about 28 MB: some 110,000 cells at 257 B per cell for nterms 11).  A
// layout that leaves the cells less than half of the array is a build error,
// caught on first use.
static_assert(kStatusRegion >= sizeof(DevStatus), "status region too small");
static_assert(kStaticBytes % 256 == 0, "array size must keep the regions 256-byte aligned");

__device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

struct Layout {
  size_t blob = 0, tmp = 0, cell = 0;
};

// Region sizes from the build's own reservation at the largest input.
int static_layout(Layout &out) {
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  Layout l;
  l.blob = up(build_blob_bytes(kStaticMaxBlobs, 1));
  l.tmp = up(build_tmp_bytes(kStaticMaxBlobs, 1));
  const size_t used = kStatusRegion + l.blob + l.tmp;
  if (used > kStaticBytes / 2) {
    note_error_text("tree2d_solve_device_static: the tree build needs more scratch per blob than the fixed "
                    "array provides for 65536 blobs");
    return TREE2D_ERR_TOO_LARGE;
  }
  l.cell = kStaticBytes - used;
  out = l;
  return TREE2D_OK;
}

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
  int mode = TREE2D_MODE_PLAIN;
  bool mirror = false;
  int rc = params_for_device_solve(p, &mode, &mirror);
  if (rc) return rc;
  // plain form only: the mixed forms and the mirror images need buffers
  // this array does not hold
  if (mode != TREE2D_MODE_PLAIN || mirror) return record_error(TREE2D_ERR_MODE);
  if (n == 0) return TREE2D_OK;
  std::lock_guard<std::mutex> lk(g_static_mu);
  Layout lay;
  rc = static_layout(lay);
  if (rc) return record_error(rc);
  unsigned char *base = nullptr;
  rc = scratch_address(&base);
  if (rc) return record_error(rc);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  Workspace ws;
  ws.status = reinterpret_cast<DevStatus *>(base);
  ws.h_status = g_host_status;
  ws.blob_arena.attach(base + kStatusRegion, lay.blob);
  ws.tmp_arena.attach(base + kStatusRegion + lay.blob, lay.tmp);
  ws.cell_arena.attach(base + kStatusRegion + lay.blob + lay.tmp, lay.cell);
  ws.init = true;  // nothing else to set up: no events, no pinned memory

  Tree t;
  rc = build_tree(ws, n, d_xy, d_cir, d_cor, p, t, s);
  if (rc == TREE2D_ERR_CUDA && (ws.blob_arena.overflowed() || ws.tmp_arena.overflowed() ||
                                ws.cell_arena.overflowed())) {
    // the arenas refuse to grow (no allocation here): the tree has more
    // cells than the cell region holds
    note_error_text("tree2d_solve_device_static: the tree has more cells than the fixed array holds");
    rc = TREE2D_ERR_TOO_LARGE;
  }
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
