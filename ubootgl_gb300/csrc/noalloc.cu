// Allocation-free multigrid solve: MG(flag) followed by one
// MG::solve(p, f, flag, h, zeroGradientBC) on device arrays, with every
// scratch buffer (the level hierarchy, the level-0 ping-pong buffer and the
// stencil codes) placed in one file-scope device array instead of memory
// from cudaMalloc.
//
// It exists for callers that must not allocate GPU memory while they run:
// code that runs under a fixed device-memory budget handed out by a host
// framework, real-time loops that must never reach the allocator (a
// cudaMalloc can synchronise the device and stall for milliseconds), or
// plug-ins whose host application owns every device allocation.  Such
// callers still pass their own input and output arrays; only the solver's
// scratch comes from here.
//
// Limits and behaviour:
//  - The scratch array is kNoAllocScratchBytes (24 MiB) on every GPU that
//    loads the library, held until the process exits.  Grids whose
//    hierarchy needs more (14 bytes per cell of the width rounded up to a
//    multiple of 32, plus about a third for the coarse levels: 1024 x 1024
//    fits, 2048 x 1024 does not) are rejected with UBG_EINVAL.
//  - All calls share the array and it keeps the last call's contents.
//    Every scratch value a solve reads is written earlier in the same solve
//    (the copy-in, the coarsening, the zero-initial-guess smoothing of the
//    coarse levels), so nothing has to be cleared and nothing carries over
//    between calls.  Calls whose work overlaps on the GPU (different streams
//    without ordering, or different host threads) race on the array.
//  - The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (host code cannot use the array's name as a device
//    pointer); make that first call before any stream capture.  A first
//    call on a capturing stream returns UBG_ESTATE without touching the
//    stream.
//  - The work is enqueued on `stream` (NULL: the legacy default stream);
//    the call returns once it is enqueued.
#include <cmath>
#include <mutex>

#include "ubg_internal.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = 24u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices] = {};

struct StateError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// Device address of the scratch array on the current device (set up once
// per device, with that device current).  The set-up is refused while `st`
// is capturing: it would end the caller's capture.
void *scratch_address(cudaStream_t st) {
  int dev = 0;
  UBG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw ubg::ArgError("device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    UBG_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone)
      throw StateError("the first allocation-free solve on a device must not be made while its "
                       "stream is capturing");
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      throw ubg::CudaError(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = ptr;
  }
  return g_scratch_ptr[dev];
}

}  // namespace

extern "C" int ubg_mg_solve_noalloc(float *p, int p_pitch, const float *f, int f_pitch,
                                    const uint8_t *flag, int flag_pitch, int width, int height,
                                    float h, int zero_gradient_bc, void *stream) {
  using namespace ubg;
  set_last_error("");
  try {
    if (!p || !f || !flag) throw ArgError("null argument");
    if (width < 8 || height < 8) throw ArgError("width and height must be >= 8");
    if (p_pitch < width || f_pitch < width || flag_pitch < width)
      throw ArgError("pitches must be at least the width");
    if (!std::isfinite(h) || !(h > 0.0f)) throw ArgError("h must be finite and > 0");
    size_t need = mg_arena_bytes(width, height);
    if (need > kNoAllocScratchBytes)
      throw ArgError("grid " + std::to_string(width) + "x" + std::to_string(height) + " needs " +
                     std::to_string(need) + " bytes of solver scratch; the allocation-free solve "
                     "has " + std::to_string(kNoAllocScratchBytes) + " bytes");
    cudaStream_t st = (cudaStream_t)stream;
    void *arena = scratch_address(st);
    MgHier mg;
    mg_bind(mg, width, height, h, arena, kNoAllocScratchBytes);
    MgLevel &L = mg.lv[0];
    size_t w4 = (size_t)width * 4, dp = (size_t)L.pitch * 4;
    UBG_CUDA(cudaMemcpy2DAsync(L.e[0], dp, p, (size_t)p_pitch * 4, w4, height,
                               cudaMemcpyDeviceToDevice, st));
    UBG_CUDA(cudaMemcpy2DAsync(L.rhs, dp, f, (size_t)f_pitch * 4, w4, height,
                               cudaMemcpyDeviceToDevice, st));
    UBG_CUDA(cudaMemcpy2DAsync(L.flag, L.pitch, flag, flag_pitch, width, height,
                               cudaMemcpyDeviceToDevice, st));
    mg.cur0 = 0;
    mg_update_fields(mg, st);  // coarse flags and stencil codes of every level
    mg_solve(mg, zero_gradient_bc != 0, st);
    UBG_CUDA(cudaMemcpy2DAsync(p, (size_t)p_pitch * 4, L.e[mg.cur0], dp, w4, height,
                               cudaMemcpyDeviceToDevice, st));
    UBG_CUDA(cudaGetLastError());
    return UBG_OK;
  } catch (const ArgError &e) {
    set_last_error(e.what());
    return UBG_EINVAL;
  } catch (const CudaError &e) {
    set_last_error(e.what());
    return UBG_ECUDA;
  } catch (const StateError &e) {
    set_last_error(e.what());
    return UBG_ESTATE;
  } catch (const std::bad_alloc &e) {
    set_last_error("out of host memory");
    return UBG_ENOMEM;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return UBG_ESTATE;
  }
}
