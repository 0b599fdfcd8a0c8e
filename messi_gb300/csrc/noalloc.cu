// noalloc.cu -- messi_inside_noalloc: the KH99 inside pass with no allocation.
//
// Some callers cannot call cudaMalloc on the path where they need Z: code
// inside a framework that owns the device allocator (and forbids side
// allocations), or real-time loops that must not enter the driver's
// allocator, whose calls can synchronise the device.  This entry point takes
// device pointers for its inputs and output, launches on the caller's stream
// and keeps its band tables in one fixed file-scope device array, so it calls
// no cudaMalloc/cudaFree and no allocating library routine.
//
// Limits.  Each of the six band tables holds at most kNoAllocCells floats,
// i.e. L * RS <= 2^20 where RS = 32 * ceil((maxspan + 1) / 32), and
// L <= kNoAllocMaxL: e.g. L = 2,048 with maxspan <= 511, or L = 1,000 with
// maxspan <= 991.  The array (about 25 MB) is reserved on every GPU that
// loads the library until the process exits.
//
// Sharing.  All calls on a device use the same array and it keeps the last
// call's contents; every cell a call reads is written by that call first (the
// band tables are filled before use, the span counter and the wavefront
// barrier are cleared).  Calls that overlap on the GPU (two streams, or two
// host threads) race on the array, so callers serialise them.
//
// Errors.  If the wavefront's bounded barrier wait gives up, the call has
// already returned MESSI_OK (the kernels run after it returns) and the only
// sign is *d_Z == NaN: callers check Z.  maxspan < 0 reads the inferred span
// back to the host and synchronises the stream once; on a stream that is
// being captured that is refused with MESSI_EINVAL.
//
// Set-up.  The first call on a device resolves the array's device address
// with cudaGetSymbolAddress while that device is current and caches it with
// the id of the device's current CUDA context; make that first call before
// any stream capture begins.  A later call in another context (after
// cudaDeviceReset, for example) resolves the address again.
#include <mutex>

#include "internal.h"

namespace messi {

constexpr size_t kNoAllocCells = size_t(1) << 20;
constexpr int kNoAllocMaxL = 16384;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    float tabs[6][kNoAllocCells];           // Lrow, Lcol, Srow, Scol, Frow, pb
    float suf[2 * (kNoAllocMaxL + 1)];      // Ssuf (+ unused outside half)
    double vec[2 * kNoAllocMaxL + 8];       // b, cb
    int maxspan[16];
    unsigned int sync[kSyncWords];          // grid-barrier words of the wavefront kernel
};

// Host code must not use this name as a device address: it is a host-side
// stand-in.  Host code reads the address with cudaGetSymbolAddress.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

static std::mutex g_noalloc_mu;
struct NoAllocSlot {
    NoAllocScratch* ptr = nullptr;
    unsigned long long ctx_id = 0;  // CUDA context the address belongs to
};
static NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices];

// Id of the calling thread's current CUDA context (0 if it cannot be read),
// through the driver entry points the runtime exposes (no libcuda link).
static unsigned long long current_context_id()
{
    typedef int (*GetCurrentFn)(void**);
    typedef int (*GetIdFn)(void*, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrentFn>(f1);
            get_id = reinterpret_cast<GetIdFn>(f2);
        }
        resolved = true;
    }
    void* c = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&c) == 0 && c && get_id(c, &id) == 0) return id;
    return 0;
}

static int noalloc_scratch(int device, NoAllocScratch** out)
{
    if (device < 0 || device >= kNoAllocMaxDevices) return MESSI_EINVAL;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocSlot& slot = g_noalloc_slot[device];
    const unsigned long long id = current_context_id();
    if (!slot.ptr || id == 0 || slot.ctx_id != id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return MESSI_ECUDA;
        slot.ptr = static_cast<NoAllocScratch*>(p);
        slot.ctx_id = id;
    }
    *out = slot.ptr;
    return MESSI_OK;
}

}  // namespace messi

using namespace messi;

extern "C" int messi_inside_noalloc(void* stream, int32_t L, const double* d_unpaired, const double* d_paired,
                                    int32_t maxspan, double B, double* d_Z)
{
    if (L < 1 || !d_unpaired || !d_paired || !d_Z) return MESSI_EINVAL;
    if (L > kNoAllocMaxL) return MESSI_ETOOBIG;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return MESSI_ECUDA;
    NoAllocScratch* s = nullptr;
    int rc = noalloc_scratch(device, &s);
    if (rc) return rc;
    messi_ctx local;  // launch bookkeeping only; owns no device memory
    local.device = device;
    local.stream = static_cast<cudaStream_t>(stream);
    int Wb = maxspan;
    if (maxspan < 0) {
        // the span is read back to the host: not possible while the stream
        // is being captured (the synchronisation would break the capture)
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(local.stream, &cs) != cudaSuccess) return MESSI_ECUDA;
        if (cs != cudaStreamCaptureStatusNone) return MESSI_EINVAL;
        if ((rc = launch_maxspan(&local, L, d_paired, s->maxspan))) return rc;
        int host = 0;
        if (cudaMemcpyAsync(&host, s->maxspan, sizeof(int), cudaMemcpyDeviceToHost, local.stream) != cudaSuccess ||
            cudaStreamSynchronize(local.stream) != cudaSuccess)
            return MESSI_ECUDA;
        Wb = host;
    }
    if (Wb > L - 1) Wb = L - 1;
    if (Wb < 0) Wb = 0;
    Band t;
    t.L = L;
    t.Wb = Wb;
    t.RS = ((Wb + 1 + 31) / 32) * 32;
    if ((size_t)L * (size_t)t.RS > kNoAllocCells) return MESSI_ETOOBIG;
    t.Lrow = s->tabs[0];
    t.Lcol = s->tabs[1];
    t.Srow = s->tabs[2];
    t.Scol = s->tabs[3];
    t.Frow = s->tabs[4];
    t.pb = s->tabs[5];
    t.Ssuf = s->suf;
    t.Osuf = s->suf + (L + 1);
    t.b = s->vec;
    t.cb = s->vec + L;
    t.u = const_cast<double*>(d_unpaired);  // read only
    t.Zd = d_Z;
    t.maxspan = s->maxspan;
    t.sync = s->sync;
    t.OSrow = t.OScol = t.OFrow = t.OFcol = t.OLrow = t.PP = t.SL = t.nrm = t.OSlast = nullptr;
    if ((rc = launch_baseline(&local, t, B))) return rc;
    if ((rc = launch_bandprep_from_dense(&local, t, d_paired, B))) return rc;
    if ((rc = run_inside(&local, t, B))) return rc;
    return MESSI_OK;
}
