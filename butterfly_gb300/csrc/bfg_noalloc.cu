// bfgFacApplyNoAlloc: the FP64 apply with its workspace in a fixed,
// statically sized device array, so the call allocates nothing.
//
// Who needs this: a caller whose GPU memory is handed out up front by
// another allocator (a framework's caching allocator that has reserved the
// device, or a fixed partition per tenant) cannot count on cudaMalloc
// succeeding, and a caller on a latency-critical loop cannot accept
// cudaMalloc/cudaFree, which may synchronise the device.  bfgFacApply sizes
// its workspace on first use and grows it with cudaMalloc; this entry point
// never does.
//
// The array below is a file-scope __device__ variable: every GPU that loads
// the library holds kNoAllocScratchBytes of it until the process exits.  In
// host code its name is only a host-side stand-in, not a device address, so
// the address is fetched with cudaGetSymbolAddress once per device (on the
// first call made with that device current) and cached.  That first call per
// device should come before any stream capture begins.
//
// All calls share the one array and it keeps the last call's contents.
// Nothing in it has to start at zero: every workspace row is written by a
// stage before any later stage or the final sum reads it.  Calls whose
// executions overlap on the GPU (other streams, other host threads) race on
// the array; callers must order them.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <climits>
#include <mutex>

#include "../../include/bfg.h"

namespace bfg {
int64_t noAllocWorkspaceEntries(bfgFac f, int64_t R, uint32_t flags);
int noAllocDevice(bfgFac f);
bfgStatus noAllocFail(bfgFac f, bfgStatus st, char const *msg);
bfgStatus noAllocApplyFp64(bfgFac f, double2 const *X, int64_t ldx, int64_t R, double2 *Y,
                           int64_t ldy, uint32_t flags, double2 *scratch);
}  // namespace bfg

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;   // 32 MiB per device
constexpr size_t kNoAllocScratchEntries = kNoAllocScratchBytes / sizeof(double2);
constexpr int kMaxDevices = 64;

__device__ __align__(256) double2 gNoAllocScratch[kNoAllocScratchEntries];

std::mutex gAddrMutex;
double2 *gAddr[kMaxDevices] = {};

}  // namespace

extern "C" bfgStatus bfgFacApplyNoAlloc(bfgFac fac, void const *X, int64_t ldx, int64_t numRhs,
                                        void *Y, int64_t ldy, uint32_t flags) {
  if (!fac) return BFG_ERROR_INVALID_ARGUMENTS;
  if (!X || !Y || numRhs < 1 || ldx < numRhs || ldy < numRhs)
    return bfg::noAllocFail(fac, BFG_ERROR_INVALID_ARGUMENTS,
                            "no-alloc apply: bad operand pointers or shapes");
  if (flags & ~BFG_APPLY_ORIGINAL_ORDER)
    return bfg::noAllocFail(fac, BFG_ERROR_INVALID_ARGUMENTS, "no-alloc apply: unknown flags");
  // entries per right-hand side first, so that a huge numRhs is refused
  // before any product can overflow
  int64_t const perRhs = bfg::noAllocWorkspaceEntries(fac, 1, flags);
  bool const tooMany = perRhs > 0 && numRhs > (int64_t)kNoAllocScratchEntries / perRhs;
  int64_t const need = tooMany ? INT64_MAX : perRhs * numRhs;
  if (need > (int64_t)kNoAllocScratchEntries) {
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "no-alloc apply: needs %lld bytes of workspace (-1: more than 2^63), the static limit is %zu bytes "
                  "(%lld right-hand sides too many; use bfgFacApply)",
                  (long long)(tooMany ? -1 : need * (int64_t)sizeof(double2)), kNoAllocScratchBytes,
                  (long long)numRhs);
    return bfg::noAllocFail(fac, BFG_ERROR_OUT_OF_RANGE, msg);
  }
  int const dev = bfg::noAllocDevice(fac);
  if (dev < 0 || dev >= kMaxDevices)
    return bfg::noAllocFail(fac, BFG_ERROR_OUT_OF_RANGE, "no-alloc apply: device index too large");
  double2 *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(gAddrMutex);
    if (!gAddr[dev]) {
      int cur = -1;
      if (cudaGetDevice(&cur) != cudaSuccess)
        return bfg::noAllocFail(fac, BFG_ERROR_CUDA, "no-alloc apply: cudaGetDevice failed");
      if (cur != dev && cudaSetDevice(dev) != cudaSuccess)
        return bfg::noAllocFail(fac, BFG_ERROR_CUDA, "no-alloc apply: cudaSetDevice failed");
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, gNoAllocScratch);
      if (cur != dev) cudaSetDevice(cur);
      if (e != cudaSuccess || !p)
        return bfg::noAllocFail(fac, BFG_ERROR_CUDA,
                                "no-alloc apply: cudaGetSymbolAddress of the static workspace failed");
      gAddr[dev] = static_cast<double2 *>(p);
    }
    scratch = gAddr[dev];
  }
  return bfg::noAllocApplyFp64(fac, static_cast<double2 const *>(X), ldx, numRhs,
                               static_cast<double2 *>(Y), ldy, flags, scratch);
}
