// Morton-pair sort that allocates nothing.
//
// Who needs it: a caller that may not call cudaMalloc -- a plugin inside a
// host application that owns all device memory through its own pool, or a
// per-frame loop that cannot take cudaMalloc's implicit device-wide
// synchronisation.  Such a caller passes device buffers for the input codes
// and the sorted output; the sort's own scratch (the second ping-pong half,
// digit histograms, look-back words and an error word) lives in the
// file-scope array below, which every GPU that loads this library keeps for
// the life of the process.
#include <cuda_runtime.h>

#include <mutex>

#include "gbt_internal.cuh"

size_t gbt_sort_static_bytes(uint32_t max_pairs);
int gbt_sort_pairs_static(cudaStream_t st, int num_sms, unsigned char *sbase, uint32_t max_pairs,
                          const uint64_t *codes_in, uint64_t *codes_out, uint32_t *idx_out, uint32_t n,
                          unsigned int **err_word);

// Scratch for GBT_NOALLOC_MAX_PAIRS pairs: 12 bytes per pair for the second
// ping-pong half, 8 passes x 1 KiB of look-back words per 4096-pair tile,
// histograms and the sort plan; about 3.6 MiB.
#define GBT_NOALLOC_SCRATCH_BYTES (4u << 20)
static __device__ __align__(256) unsigned char g_sort_scratch[GBT_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_lock;
unsigned char *g_addr[kMaxDevices] = {};  // device address of g_sort_scratch, per device
int g_sms[kMaxDevices] = {};
}  // namespace

extern "C" int gbt_sort_morton_pairs_noalloc(void *stream, const uint64_t *d_codes_in, uint64_t *d_codes_out,
                                             uint32_t *d_idx_out, uint32_t n) {
    if (n == 0) return GBT_OK;
    if (!d_codes_in || !d_codes_out || !d_idx_out) return GBT_EINVAL;
    if (n > GBT_NOALLOC_MAX_PAIRS) return GBT_EINVAL;  // larger sorts need gbt_lbvh_build's allocated scratch
    if (gbt_sort_static_bytes(GBT_NOALLOC_MAX_PAIRS) > GBT_NOALLOC_SCRATCH_BYTES) return GBT_EUNSUPPORTED;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GBT_ECUDA;
    unsigned char *base;
    int sms;
    {
        // first call on this device: look up the array's device address with
        // the device current (the host-side symbol is not a device address)
        std::lock_guard<std::mutex> g(g_lock);
        if (!g_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_sort_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return GBT_ECUDA;
            }
            int s = 0;
            if (cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || s <= 0) return GBT_ECUDA;
            g_sms[dev] = s;
            g_addr[dev] = static_cast<unsigned char *>(p);
        }
        base = g_addr[dev];
        sms = g_sms[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned int *err = nullptr;
    int rc = gbt_sort_pairs_static(st, sms, base, GBT_NOALLOC_MAX_PAIRS, d_codes_in, d_codes_out, d_idx_out, n, &err);
    if (rc) return rc;
    unsigned int flags = 0;
    if (cudaMemcpyAsync(&flags, err, sizeof(flags), cudaMemcpyDeviceToHost, st) != cudaSuccess) return GBT_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return GBT_ECUDA;
    if (flags & GBT_DEVERR_SPIN) return GBT_ETIMEOUT;
    return flags ? GBT_EDEVICE : GBT_OK;
}
