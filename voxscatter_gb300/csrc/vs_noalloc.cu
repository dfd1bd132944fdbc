// Allocation-free operator apply.
//
// Some callers cannot allocate device memory at the moment they need a matvec:
// services that reserve all their device memory at start-up and forbid
// allocation afterwards, and MEX or plug-in hosts that run the solver inside a
// device-memory budget owned by another allocator (MATLAB's GPU memory pool,
// a framework's caching allocator), where a cudaMalloc of the library's own
// either fails or competes with the host.  vs_op_apply_device allocates its
// pipeline intermediates on demand; this entry point instead runs the same
// fused pipeline with its intermediates in one statically sized device array
// that the library owns.
//
// The array is kNoAllocScratchBytes (64 MiB) of file-scope __device__ memory:
// every GPU that loads the library holds it until the process exits.  Its
// device address is looked up once per device (cudaGetSymbolAddress), by the
// first call made with that device current, and cached for the life of the
// process: this assumes the device's primary context is not reset
// (cudaDeviceReset) while the library is in use.  Make that first call before
// any stream capture.  All calls share the array and it keeps the last call's
// contents; the pipeline writes every scratch element before reading it, so
// nothing needs clearing.  Two calls whose work overlaps on the GPU (other
// streams, other host threads) race on the array: serialise them.
#include "vs_internal.h"

#include <mutex>

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.
void* scratch_address(int device) {
  VS_REQUIRE(device >= 0 && device < kMaxDevices, "device index out of range");
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
      throw vs::Error(VS_ERR_CUDA, std::string("cudaGetSymbolAddress(noalloc scratch): ") + cudaGetErrorString(e));
    g_addr[device] = ptr;
  }
  return g_addr[device];
}

}  // namespace

extern "C" int vs_op_apply_device_noalloc(vs_op* op, const void* x, void* y, int64_t nrhs, int mode, int precision) {
  if (!op) return VS_ERR_ARG;
  try {
    vs_ctx* ctx = op->ctx;
    VS_CUDA(cudaSetDevice(ctx->device));
    VS_REQUIRE(x && y, "NULL argument");
    VS_REQUIRE(nrhs >= 1 && nrhs <= 65535, "nrhs must be in [1, 65535]");
    VS_REQUIRE(precision == VS_C64 || precision == VS_C128, "precision must be VS_C64 or VS_C128");
    VS_REQUIRE(mode >= VS_NOTRANSP && mode <= VS_CONJTRANSP, "bad mode");
    const size_t esz = precision == VS_C64 ? sizeof(float2) : sizeof(double2);
    const size_t n1 = (size_t)op->P * op->M * op->N * 3 * nrhs;
    const size_t n2 = (size_t)op->P * op->Q * op->N * 3 * nrhs;
    const size_t off2 = (n1 * esz + 255) / 256 * 256;
    const size_t need = off2 + n2 * esz;
    if (need > kNoAllocScratchBytes)
      throw vs::Error(VS_ERR_UNSUPPORTED, "vs_op_apply_device_noalloc needs " + std::to_string(need) +
                                              " bytes of scratch; the static limit is " +
                                              std::to_string(kNoAllocScratchBytes) + " bytes (64 MiB)");
    unsigned char* base = static_cast<unsigned char*>(scratch_address(ctx->device));
    cudaStream_t st = ctx->stream;
    if (precision == VS_C64)
      vs::matvec_scratch<float>(*op, (const float2*)x, (float2*)y, (int)nrhs, mode, (float2*)base,
                                (float2*)(base + off2), st);
    else
      vs::matvec_scratch<double>(*op, (const double2*)x, (double2*)y, (int)nrhs, mode, (double2*)base,
                                 (double2*)(base + off2), st);
    return VS_OK;
  } catch (const vs::Error& e) {
    record_error(op->ctx, e.what());
    return e.status;
  } catch (const std::exception& e) {
    record_error(op->ctx, e.what());
    return VS_ERR_CUDA;
  }
}
