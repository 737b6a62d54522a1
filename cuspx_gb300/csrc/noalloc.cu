// noalloc.cu -- signing with no device allocation by this library.
//
// Who needs it: a caller that must not allocate device memory while it runs.
// cudaMalloc / cudaFree take process-wide driver locks and cudaFree waits for
// the whole device, which stalls every other stream -- unacceptable inside a
// latency-critical serving loop; and some hosts (plugins inside a larger
// application, engines with a fixed device-memory budget) own all device
// memory through their own allocator and forbid a library from allocating
// behind their back.  Such a caller allocates its inputs and outputs itself
// and calls cuspx_sign_noalloc; the signing pipeline's scratch comes from a
// fixed array that lives in this library's device image.
//
// The array is 8 MiB per GPU that loads the library, held until the process
// exits.  It is shared by every call: calls that overlap on the GPU (two
// streams, two host threads) race on it and must be serialised by the
// caller.  Nothing in it has to start at zero -- every scratch value a kernel
// reads was written earlier in the same call -- so it is never cleared.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/cuspx.h"
#include "spx_launch.cuh"
#include "spx_sets.h"

namespace cuspx {
void ensure_registered();
SetParams make_params(const SetDesc &s);
}  // namespace cuspx
using namespace cuspx;

#define CUSPX_NOALLOC_SCRATCH_BYTES (8u << 20)

// Device scratch of the no-allocation entry point.  In host code this name
// is only a stand-in for the device symbol: its device address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) uint8_t g_noalloc_scratch[CUSPX_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;

struct DeviceSetup {
    bool ready = false;
    uint8_t *scratch = nullptr;   // device address of g_noalloc_scratch
    bool configured[2][3][2] = {};
};

DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

// scratch bytes for `count` signatures of P, carved in five 256-aligned pieces
size_t scratch_bytes(const SetParams &P, size_t count) {
    const size_t n = P.n;
    return up256(count * sizeof(SignWork)) + up256(count * P.k * n) +
           up256(count * P.d * ((size_t)1 << P.hp) * n) + up256(count * P.d * n) +
           up256(count * P.d * P.len * 16 * n);
}

}  // namespace

extern "C" int cuspx_sign_noalloc(int set, size_t count, const uint8_t *d_sks, const uint8_t *d_msgs,
                                  const uint64_t *d_msg_off, const uint64_t *d_msg_len, const uint8_t *d_optrand,
                                  uint8_t *d_sigs, int32_t *d_status, void *stream) {
    if (set < 0 || set >= kNumSets) return CUSPX_EINVAL;
    if (count == 0) return CUSPX_OK;
    if (!d_sks || !d_msgs || !d_msg_off || !d_msg_len || !d_sigs || !d_status) return CUSPX_EINVAL;
    // The kernels move keys, optrand, signatures, offsets and lengths as
    // 8-byte words and read messages as 16-byte vectors; a misaligned
    // pointer would fault on the device (and leave the context unusable),
    // so it is refused here before anything is launched.
    auto misaligned = [](const void *p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) != 0; };
    if (misaligned(d_sks, 8) || misaligned(d_sigs, 8) || misaligned(d_optrand, 8) || misaligned(d_msg_off, 8) ||
        misaligned(d_msg_len, 8) || misaligned(d_msgs, 16) || misaligned(d_status, 4))
        return CUSPX_EINVAL;
    const SetDesc &sd = kSets[set];
    const SetParams P = make_params(sd);
    if (count > (1u << 20) || scratch_bytes(P, count) > CUSPX_NOALLOC_SCRATCH_BYTES) return CUSPX_ETOOBIG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return CUSPX_ECUDA;
    ensure_registered();
    const FamilyOps &ops = g_family[sd.hash][sd.n / 8 - 2][sd.robust];
    {
        // first call on this device (with it current): resolve the array's
        // device address and set the kernels' shared-memory limits
        std::lock_guard<std::mutex> lk(g_setup_mu);
        DeviceSetup &ds = g_setup[dev];
        if (!ds.ready) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CUSPX_ECUDA;
            ds.scratch = (uint8_t *)p;
            ds.ready = true;
        }
        bool &cfg = ds.configured[sd.hash][sd.n / 8 - 2][sd.robust];
        if (!cfg) {
            if (ops.configure() != cudaSuccess) return CUSPX_ECUDA;
            cfg = true;
        }
    }
    uint8_t *base = g_setup[dev].scratch;
    const size_t n = P.n;
    SignArgs A;
    A.count = (uint32_t)count;
    A.sk = KeyRef{d_sks, nullptr, (uint32_t)P.sk_bytes};
    A.msg = MsgRef{d_msgs, d_msg_off, d_msg_len};
    A.optrand = d_optrand;
    A.sig = d_sigs;
    A.status = d_status;
    A.work = (SignWork *)base;
    base += up256(count * sizeof(SignWork));
    A.fors_roots = base;
    base += up256(count * P.k * n);
    A.leaves = base;
    base += up256(count * P.d * ((size_t)1 << P.hp) * n);
    A.roots = base;
    base += up256(count * P.d * n);
    A.chains = base;
    Tuning tu;   // the default mapping: any mapping gives the same bytes
    ops.sign(P, A, tu, (cudaStream_t)stream, nullptr, 0, nullptr);
    return cudaGetLastError() == cudaSuccess ? CUSPX_OK : CUSPX_ECUDA;
}
