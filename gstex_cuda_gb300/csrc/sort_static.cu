// Pair sort for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a render loop running
// inside a host framework that owns every device allocation through its own
// pool, a plugin that is handed only a stream and raw pointers, or real-time
// code that must not let an allocation synchronise the device or fail in the
// middle of a frame.  gstex_sort_pairs needs a caller-provided workspace; this
// variant keeps its scratch in one file-scope device array instead, so the
// caller passes only its inputs and outputs.
//
// The array is sized for GSTEX_SORT_STATIC_MAX_ITEMS pairs (13.1 MB) and
// exists on every GPU that loads the library until the process exits.  The
// first call in each CUDA context looks up the array's device address, so it
// should come before any stream capture.  All
// calls on a device share it and it keeps the last call's contents; the sort
// writes every scratch word before reading it, so nothing has to be cleared
// between calls.  Calls that overlap on the GPU (other streams or host
// threads on the same device) race on the array and must be serialised by the
// caller.
#include <mutex>

#include "common.cuh"

namespace gstex {

// Scratch of gstex_sort_pairs at GSTEX_SORT_STATIC_MAX_ITEMS pairs: alternate
// keys (8 B/pair) + alternate values (4 B/pair) + 256 digit counters for each
// of 512 blocks + 256 digit totals.
constexpr size_t kStaticScratchBytes = (size_t)GSTEX_SORT_STATIC_MAX_ITEMS * 8 +
                                       (size_t)GSTEX_SORT_STATIC_MAX_ITEMS * 4 + 256 * 512 * 4 + 256 * 4;

static __device__ __align__(256) unsigned char g_sort_scratch[kStaticScratchBytes];

namespace {
// The array's device address belongs to the CUDA context the module was
// loaded into, so it is cached per context: keyed by the context's unique id
// (cuCtxGetId, which is never reused, unlike a context handle after a device
// reset), resolved through the runtime so that the library does not link the
// driver library.  Without those entry points the address is looked up on
// every call.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
constexpr int kCacheSlots = 64;
std::mutex g_scratch_mutex;
bool g_driver_resolved = false;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
unsigned long long g_cache_ctx[kCacheSlots] = {};
void* g_cache_ptr[kCacheSlots] = {};
int g_cache_next = 0;

// Id of the calling thread's current context; false when there is none yet
// or the driver entry points are unavailable.  Called with the mutex held.
bool current_context_id(unsigned long long* id) {
    if (!g_driver_resolved) {
        g_driver_resolved = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            g_ctx_get_current = (CtxGetCurrentFn)f1;
            g_ctx_get_id = (CtxGetIdFn)f2;
        }
        cudaGetLastError();  // a failed lookup leaves no sticky error
    }
    if (!g_ctx_get_current || !g_ctx_get_id) return false;
    void* ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0 || !ctx) return false;
    return g_ctx_get_id(ctx, id) == 0;
}
}  // namespace

// Device address of g_sort_scratch in the current context.  In host code the
// array's name is only a host-side stand-in, so the address is looked up
// (which also makes the runtime's context current) the first time a context
// calls, and cached under that context's id.
static int static_scratch(void** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    if (have_id) {
        for (int i = 0; i < kCacheSlots; i++)
            if (g_cache_ptr[i] && g_cache_ctx[i] == id) {
                *out = g_cache_ptr[i];
                return GSTEX_OK;
            }
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || !p) {
        set_cuda_error(e, "sort_pairs_static: cudaGetSymbolAddress");
        return GSTEX_ERR_CUDA;
    }
    if (!have_id) have_id = current_context_id(&id);
    if (have_id) {
        g_cache_ctx[g_cache_next] = id;
        g_cache_ptr[g_cache_next] = p;
        g_cache_next = (g_cache_next + 1) % kCacheSlots;
    }
    *out = p;
    return GSTEX_OK;
}

}  // namespace gstex

extern "C" int gstex_sort_pairs_static(int n, int end_bit, const int64_t* keys_in, const int32_t* vals_in,
                                       int64_t* keys_out, int32_t* vals_out, gstex_stream_t stream) {
    if (n < 0 || end_bit < 0 || end_bit > 64) return GSTEX_ERR_INVALID_ARGUMENT;
    if (n > GSTEX_SORT_STATIC_MAX_ITEMS) return GSTEX_ERR_CAPACITY;
    const size_t need = gstex_sort_workspace_bytes(n);
    if (need > gstex::kStaticScratchBytes) return GSTEX_ERR_CAPACITY;
    if (n == 0) return GSTEX_OK;
    void* scratch = nullptr;
    const int rc = gstex::static_scratch(&scratch);
    if (rc) return rc;
    return gstex_sort_pairs(n, end_bit, keys_in, vals_in, keys_out, vals_out, scratch, gstex::kStaticScratchBytes,
                            stream);
}
