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
// exists on every GPU that loads the library until the process exits.  All
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
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_ptr[kMaxDevices] = {};
}  // namespace

// Device address of g_sort_scratch on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up once
// per device (with that device current) and cached.
static int static_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_cuda_error(e, "sort_pairs_static: cudaGetDevice"); return GSTEX_ERR_CUDA; }
    if (dev < 0 || dev >= kMaxDevices) return GSTEX_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess || !p) {
            set_cuda_error(e, "sort_pairs_static: cudaGetSymbolAddress");
            return GSTEX_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
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
