// noalloc.cu -- one inner-product round that allocates no memory.
//
// Every other entry point of this library allocates device memory (tables,
// per-prover scratch, proof buffers) through the stream-ordered allocator.
// Some callers cannot allow that: a prover embedded in a larger proving
// system whose memory manager has already reserved (nearly) all HBM for its
// own pool, where a cudaMalloc would fail or fragment that pool, and callers
// that issue work on a stream shared with latency-critical work, where a
// device-synchronising cudaMalloc/cudaFree would stall everything else.
// effsc_ip_round_noalloc serves them: the caller passes the tables and every
// output in its own device memory, and the only scratch -- the per-block
// partial sums of the grid reduction, the round result and the block
// counter -- lives in the file-scope array below, which every GPU that loads
// the library holds until the process exits.
#include "effsc_gpu.h"
#include "kernels.h"

#include <mutex>

using namespace effsc;

namespace {

constexpr int NOALLOC_MAX_BLOCKS = 4096;
constexpr size_t NOALLOC_RESULT = (size_t)NOALLOC_MAX_BLOCKS * 12;   // 15 result words follow the partials
constexpr size_t NOALLOC_COUNTER = NOALLOC_RESULT + 16;              // then one u32 block counter
constexpr size_t NOALLOC_WORDS = NOALLOC_COUNTER + 2;

// 4096 blocks x 12 words of partial sums + 16 result words + counter: 393,360 bytes.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[NOALLOC_WORDS];

constexpr int MAX_DEVICES = 64;
u64* g_scratch_dev[MAX_DEVICES];   // device address of g_noalloc_scratch, per device
std::mutex g_setup_mu;

// Resolve the array's device address on the current device (once per device).
// The host-side name g_noalloc_scratch is only a stand-in: never pass it to a kernel.
int scratch_for_device(int dev, u64** out) {
    if (dev < 0 || dev >= MAX_DEVICES) return effsc_set_error(EFFSC_INVALID_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_dev[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return effsc_set_error(EFFSC_CUDA_ERROR, "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
        kernels_init(dev);
        g_scratch_dev[dev] = (u64*)p;
    }
    *out = g_scratch_dev[dev];
    return EFFSC_OK;
}

}  // namespace

extern "C" int effsc_ip_round_noalloc(const uint64_t* a, const uint64_t* b, uint64_t* a_out, uint64_t* b_out,
                                      size_t len, const uint64_t* challenge, uint64_t* out_evals, int blocks,
                                      void* stream) {
    if (!a || !b || !out_evals) return effsc_set_error(EFFSC_INVALID_ARG, "NULL table or output pointer");
    if (blocks < 0 || blocks > NOALLOC_MAX_BLOCKS)
        return effsc_set_error(EFFSC_INVALID_ARG,
                               "blocks = %d exceeds the no-alloc scratch capacity of %d blocks", blocks, NOALLOC_MAX_BLOCKS);
    if (challenge) {
        if (!a_out || !b_out) return effsc_set_error(EFFSC_INVALID_ARG, "a_out/b_out are NULL");
        if (len < 4 || (len & (len - 1)))
            return effsc_set_error(EFFSC_INVALID_ARG, "len = %zu: a folding round needs a power of two >= 4", len);
    } else if (len < 1) {
        return effsc_set_error(EFFSC_INVALID_ARG, "len = 0");
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "cudaGetDevice: %s", cudaGetErrorString(e));
    u64* scratch = nullptr;
    int rc = scratch_for_device(dev, &scratch);
    if (rc != EFFSC_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;

    RoundArgs args;
    memset(&args, 0, sizeof args);
    const u64* tabs[2] = {(const u64*)a, (const u64*)b};
    u64* outs[2] = {(u64*)a_out, (u64*)b_out};
    for (int t = 0; t < 2; t++)
        for (int c = 0; c < 3; c++) {
            args.t[t].in[c] = tabs[t] + c * len;
            args.t[t].out[c] = outs[t] ? outs[t] + c * len : nullptr;
        }
    args.L = len;
    if (challenge)
        for (int c = 0; c < 3; c++) args.chal[c] = challenge[c] >= 0xFFFFFFFF00000001ULL ? challenge[c] - 0xFFFFFFFF00000001ULL : challenge[c];
    args.partials = scratch;
    args.result = scratch + NOALLOC_RESULT;
    args.counter = (u32*)(scratch + NOALLOC_COUNTER);
    // the last block of a call resets the counter; clear it anyway in case an
    // earlier call on this device did not complete
    e = cudaMemsetAsync(args.counter, 0, sizeof(u32), s);
    if (e != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    u64 work = challenge ? len / 4 : (len > 1 ? len / 2 : 1);
    int grid = blocks;
    if (!grid) {
        u64 g = (work + KERNEL_TPB - 1) / KERNEL_TPB;
        u64 mg = (u64)max_grid();
        grid = (int)(g < 1 ? 1 : (g < mg ? g : mg));
    }
    bool ok = challenge ? launch_fused(POL_IP, SEM_MSB_PAD, 3u, true, args, grid, s)
                        : launch_eval(POL_IP, SEM_MSB_PAD, 3u, args, grid, s);
    if (!ok) return effsc_set_error(EFFSC_UNSUPPORTED, "no kernel for the no-alloc round");
    e = cudaGetLastError();
    if (e != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "no-alloc round launch: %s", cudaGetErrorString(e));
    e = cudaMemcpyAsync(out_evals, scratch + NOALLOC_RESULT, 6 * sizeof(u64), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return effsc_set_error(EFFSC_CUDA_ERROR, "cudaMemcpyAsync: %s", cudaGetErrorString(e));
    return EFFSC_OK;
}
