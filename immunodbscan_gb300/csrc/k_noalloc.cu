// k_noalloc.cu -- exact-duplicate collapse that allocates no device memory.
//
// Some callers of this library cannot allocate device memory: a host whose
// device memory is owned by another allocator (a framework's caching pool that
// has reserved the GPU), or a latency-bound serving loop in which cudaMalloc /
// cudaFree -- which synchronise the whole device -- are not allowed.  For them,
// idb_dedupe_noalloc runs the duplicate-collapse step of the clustering path
// (rule S3: equal length, equal V and J bitsets, equal bytes; the minimum row of
// a class represents it and carries the class size) with its hash table in a
// fixed array that is part of the library image instead of in allocated memory.
//
// The scratch array is a file-scope __device__ variable: every GPU that loads
// the library holds it (about 5 MB) until the process exits.  It is shared by
// all calls on a device and keeps the last call's contents, so each call first
// resets it; two calls that overlap on the GPU race on it and must be
// serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/immunodbscan_gb300.h"
#include "bitops.cuh"

namespace idb {
void set_last_error(const char *msg);
}

namespace {

constexpr uint32_t kMaxRows = IDB_DEDUPE_NOALLOC_MAX_ROWS;
constexpr uint32_t kSlots = 2 * kMaxRows;          // power of two, load factor <= 1/2
constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr uint32_t kMaxDevices = 64;

struct NoAllocScratch {
    uint32_t table[kSlots];    // row index of a class member (minimum after the pass)
    uint32_t count[kSlots];    // class sizes
    uint32_t slot[kMaxRows];   // slot of every row
    uint32_t error;            // non-zero: a probe sequence exceeded its bound
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch, resolved once per device.
NoAllocScratch *g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

struct Args {
    const uint8_t *seq;
    const int64_t *off;
    const uint64_t *vbits, *jbits;
    uint32_t VW, JW;
    uint32_t n;
    NoAllocScratch *scr;
};

__global__ void k_noalloc_reset(NoAllocScratch *scr, uint32_t slots) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += stride) {
        scr->table[i] = kEmpty;
        scr->count[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) scr->error = 0;
}

__device__ bool same_row(const Args &a, uint32_t x, uint32_t y) {
    const int64_t ox = a.off[x], oy = a.off[y];
    const uint32_t lx = (uint32_t)(a.off[x + 1] - ox);
    if ((uint32_t)(a.off[y + 1] - oy) != lx) return false;
    if (a.vbits)
        for (uint32_t w = 0; w < a.VW; ++w)
            if (a.vbits[(size_t)x * a.VW + w] != a.vbits[(size_t)y * a.VW + w]) return false;
    if (a.jbits)
        for (uint32_t w = 0; w < a.JW; ++w)
            if (a.jbits[(size_t)x * a.JW + w] != a.jbits[(size_t)y * a.JW + w]) return false;
    for (uint32_t k = 0; k < lx; ++k)
        if (a.seq[ox + k] != a.seq[oy + k]) return false;
    return true;
}

__global__ void k_noalloc_insert(Args a, uint32_t mask) {
    NoAllocScratch *scr = a.scr;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const int64_t o = a.off[i];
        const uint32_t L = (uint32_t)(a.off[i + 1] - o);
        uint64_t h = idb::mix64(0xD1B54A32D192ED03ull, L);
        if (a.vbits)
            for (uint32_t w = 0; w < a.VW; ++w) h = idb::mix64(h, a.vbits[(size_t)i * a.VW + w]);
        if (a.jbits)
            for (uint32_t w = 0; w < a.JW; ++w) h = idb::mix64(h, a.jbits[(size_t)i * a.JW + w]);
        uint64_t word = 0;
        for (uint32_t k = 0; k < L; ++k) {
            word = (word << 8) | a.seq[o + k];
            if ((k & 7) == 7) { h = idb::mix64(h, word); word = 0; }
        }
        h = idb::mix64(h, word);
        uint32_t s = (uint32_t)h & mask;
        uint32_t it = 0;
        for (;; ++it) {
            if (it > mask) {                // the table cannot fill at load <= 1/2
                atomicOr(&scr->error, 1u);
                s = kEmpty;
                break;
            }
            uint32_t cur = *((volatile uint32_t *)&scr->table[s]);
            if (cur == kEmpty) {
                const uint32_t prev = atomicCAS(&scr->table[s], kEmpty, i);
                if (prev == kEmpty) break;
                cur = prev;
            }
            if (same_row(a, i, cur)) {
                atomicMin(&scr->table[s], i);
                break;
            }
            s = (s + 1) & mask;
        }
        scr->slot[i] = s;
        if (s != kEmpty) atomicAdd(&scr->count[s], 1u);
    }
}

__global__ void k_noalloc_final(uint32_t n, const NoAllocScratch *scr, uint32_t *rep_out,
                                uint32_t *copies_out) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t s = scr->slot[i];
        const uint32_t r = s == kEmpty ? i : scr->table[s];
        rep_out[i] = r;
        copies_out[i] = r == i ? (s == kEmpty ? 1u : scr->count[s]) : 0u;
    }
}

idb_status fail(idb_status st, const char *msg) {
    idb::set_last_error(msg);
    return st;
}

}  // namespace

extern "C" idb_status idb_dedupe_noalloc(const char *seqs, const int64_t *seq_offsets,
                                         const uint64_t *v_bits, uint32_t v_words,
                                         const uint64_t *j_bits, uint32_t j_words,
                                         uint32_t n_rows, uint32_t *rep_out, uint32_t *copies_out,
                                         void *stream) {
    if (n_rows == 0) return IDB_OK;
    if (!seqs || !seq_offsets || !rep_out || !copies_out)
        return fail(IDB_ERR_INVALID_ARG, "idb_dedupe_noalloc: NULL input or output pointer");
    if (n_rows > kMaxRows)
        return fail(IDB_ERR_UNSUPPORTED,
                    "idb_dedupe_noalloc: n_rows exceeds IDB_DEDUPE_NOALLOC_MAX_ROWS (262144)");
    if ((v_bits && v_words == 0) || (j_bits && j_words == 0) || v_words > 8 || j_words > 8)
        return fail(IDB_ERR_INVALID_ARG, "idb_dedupe_noalloc: bitset word counts must be 1..8");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= (int)kMaxDevices) {
        cudaGetLastError();
        return fail(IDB_ERR_NO_DEVICE, "idb_dedupe_noalloc: no current CUDA device");
    }
    NoAllocScratch *scr = nullptr;
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return fail(IDB_ERR_CUDA, "idb_dedupe_noalloc: cudaGetSymbolAddress failed");
            }
            g_scratch_addr[dev] = static_cast<NoAllocScratch *>(p);
        }
        scr = g_scratch_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaGetLastError();
    uint32_t slots = 1024;
    while (slots < 2 * n_rows) slots <<= 1;      // <= kSlots because n_rows <= kMaxRows
    Args a;
    a.seq = reinterpret_cast<const uint8_t *>(seqs);
    a.off = seq_offsets;
    a.vbits = v_bits;
    a.jbits = j_bits;
    a.VW = v_words;
    a.JW = j_words;
    a.n = n_rows;
    a.scr = scr;
    const int threads = 256;
    const int grid_rows = (int)((n_rows + threads - 1) / threads);
    const int grid_slots = (int)((slots + threads - 1) / threads);
    k_noalloc_reset<<<grid_slots, threads, 0, s>>>(scr, slots);
    k_noalloc_insert<<<grid_rows, threads, 0, s>>>(a, slots - 1);
    k_noalloc_final<<<grid_rows, threads, 0, s>>>(n_rows, scr, rep_out, copies_out);
    if (cudaGetLastError() != cudaSuccess)
        return fail(IDB_ERR_CUDA, "idb_dedupe_noalloc: kernel launch failed");
    uint32_t err = 0;
    if (cudaMemcpyAsync(&err, &scr->error, sizeof err, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return fail(IDB_ERR_CUDA, "idb_dedupe_noalloc: stream failed");
    }
    if (err) return fail(IDB_ERR_DEVICE_STALL, "idb_dedupe_noalloc: hash probe bound reached");
    return IDB_OK;
}
