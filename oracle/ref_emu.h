// ref_emu.h -- TEST INFRASTRUCTURE: a host execution model for the reference's
// own CUDA translation unit (cuda/Interlink.cu and the headers it includes),
// so that the reference's clustering path runs on CPU cores and its answers
// can pin the oracle (oracle/oracle.cpp).  Nothing in the product links this.
//
// oracle/build_ref.py streams the reference's sources from their place in the
// reference tree into g++ with this header force-included.  The sources are
// not modified except for the kernel-launch syntax, which g++ cannot parse:
//     kernel<<<grid, block[, shmem]>>>(args);
// is read as
//     ::emu::launch("kernel", ::emu::Config(grid, block[, shmem]), [&]() { kernel(args); });
// Under g++ the CUDA headers define __global__, __device__, __host__ and
// __shared__ as nothing, so kernels are plain function templates and
// "extern __shared__ int s[]" names one global array per name (s, cs below).
//
// Execution model (ref_emu.cpp):
//  * every kernel of the path except find_string_occurences is written as a
//    grid-stride loop whose block-level helpers stride over threadIdx.x
//    (cuda/PSDBSCAN.hcu:129-177, 525-931; cuda/BitsetVector.inl:214-314).  Such
//    a kernel is run as one block of one thread, which visits every iteration of
//    its loops in order: one of the interleavings the GPU may produce.  Barriers
//    in it complete at once, __syncthreads_count returns the caller's own value.
//  * find_string_occurences (cuda/BitsetVector.inl:118-176) gives each thread
//    one position of the query and combines them with __syncthreads_count, so it
//    runs with its real geometry: one block per row, blockDim.x threads, each
//    thread a fiber (ucontext) and every barrier a rendezvous of the block's
//    live fibers.
//  * atomics are plain read-modify-writes (one OS thread runs everything).
//  * the CUDA runtime calls of the path (device properties, cudaMalloc/Memcpy/
//    Free, synchronise, memory info) act on host memory.
#pragma once

#include <cstddef>
#include <cstdio>
#include <functional>

#include <thrust/device_vector.h>
#include <thrust/host_vector.h>
#include <thrust/functional.h>
#include <thrust/sort.h>   // used without an include at cuda/PSDBSCAN.hcu:1081,1274

// Thrust in this toolkit no longer has unary_function / binary_function /
// identity, which the reference's headers name (cuda/SpecialFunctors.hcu:73 and
// others, cuda/PSDBSCAN.hcu:1108,1194).  Stand-ins with the old meaning:
namespace thrust {
template <class A, class R> struct unary_function { typedef A argument_type; typedef R result_type; };
template <class A1, class A2, class R> struct binary_function {
    typedef A1 first_argument_type; typedef A2 second_argument_type; typedef R result_type;
};
template <class T> struct identity {
    typedef T argument_type;
    typedef T result_type;
    const T &operator()(const T &x) const { return x; }
};
}  // namespace thrust

// nvcc includes cuda_runtime.h in every translation unit; its typed
// cudaMalloc overload is what cuda/BitsetVector.inl:191 calls.
template <class T> inline cudaError_t cudaMalloc(T **p, size_t n) { return ::cudaMalloc((void **)p, n); }

namespace emu {

struct Config {
    dim3 grid, block;
    size_t shmem;
    Config(dim3 g, dim3 b, size_t s = 0) : grid(g), block(b), shmem(s) {}
};

// Built-in index variables of the thread being run.
extern uint3 thread_idx, block_idx;
extern dim3 block_dim, grid_dim;

void launch(const char *name, const Config &cfg, std::function<void()> body);
void syncthreads();
int syncthreads_count(int pred);

}  // namespace emu

#define threadIdx ::emu::thread_idx
#define blockIdx ::emu::block_idx
#define blockDim ::emu::block_dim
#define gridDim ::emu::grid_dim
#define __syncthreads() ::emu::syncthreads()
#define __syncthreads_count(p) ::emu::syncthreads_count(p)

// Dynamic shared memory of the path's kernels ("extern __shared__ int s[]",
// cuda/BitsetVector.inl:133; "extern __shared__ int cs[]", cuda/PSDBSCAN.hcu:767,
// :857): one block runs at a time, so one host array per name serves them all.
extern int s[];
extern int cs[];

// Atomics: one OS thread runs every emulated thread, so plain updates suffice.
template <class T, class U> inline T atomicAdd(T *p, U v) { T o = *p; *p = (T)(o + v); return o; }
template <class T, class U> inline T atomicOr(T *p, U v) { T o = *p; *p = (T)(o | v); return o; }
template <class T, class U> inline T atomicExch(T *p, U v) { T o = *p; *p = (T)v; return o; }
template <class T, class U, class V> inline T atomicCAS(T *p, U cmp, V v) {
    T o = *p;
    if (o == (T)cmp) *p = (T)v;
    return o;
}

// Device min/max on int and unsigned (cuda/PSDBSCAN.hcu:250, 282).
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
