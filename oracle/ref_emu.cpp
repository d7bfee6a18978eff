// ref_emu.cpp -- TEST INFRASTRUCTURE: the host execution model declared in
// ref_emu.h (kernel launches, barriers, CUDA runtime calls on host memory) for
// the reference's own CUDA translation unit.  See ref_emu.h for the model.
#include "ref_emu.h"

#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include <ucontext.h>

#include <cuda_runtime_api.h>

int s[1 << 16];
int cs[1 << 16];

namespace emu {

uint3 thread_idx, block_idx;
dim3 block_dim, grid_dim;

namespace {

// One block of fibers in lockstep at its barriers.
struct Fiber {
    ucontext_t ctx;
    uint3 tid;
    bool done = false;
    bool waiting = false;   // arrived at the current barrier
    int pred = 0;
    int result = 0;
};

struct Block {
    ucontext_t sched;
    std::vector<Fiber> fibers;
    std::function<void()> *body = nullptr;
    int current = -1;
};

Block *g_block = nullptr;   // the block being run with fibers (nullptr: one thread)

// Fiber stacks, allocated once and reused by every block (not cleared).
const size_t kStack = 256 * 1024;
std::vector<std::unique_ptr<char[]>> g_stacks;
char *stack_of(unsigned t) {
    while (g_stacks.size() <= t) g_stacks.emplace_back(new char[kStack]);
    return g_stacks[t].get();
}

void fiber_entry(unsigned lo, unsigned hi) {
    uintptr_t p = ((uintptr_t)hi << 32) | (uintptr_t)lo;
    Block *b = reinterpret_cast<Block *>(p);
    Fiber &f = b->fibers[b->current];
    (*b->body)();
    f.done = true;
    swapcontext(&f.ctx, &b->sched);   // never resumed
}

void set_thread(const uint3 &t) { thread_idx = t; }

void run_block_fibers(const Config &cfg, std::function<void()> &body) {
    const unsigned nt = cfg.block.x * cfg.block.y * cfg.block.z;
    Block b;
    b.body = &body;
    b.fibers.resize(nt);
    uintptr_t bp = reinterpret_cast<uintptr_t>(&b);
    for (unsigned t = 0; t < nt; ++t) {
        Fiber &f = b.fibers[t];
        f.tid = uint3{t % cfg.block.x, (t / cfg.block.x) % cfg.block.y, t / (cfg.block.x * cfg.block.y)};
        getcontext(&f.ctx);
        f.ctx.uc_stack.ss_sp = stack_of(t);
        f.ctx.uc_stack.ss_size = kStack;
        f.ctx.uc_link = nullptr;
        makecontext(&f.ctx, (void (*)())fiber_entry, 2, (unsigned)(bp & 0xffffffffu),
                    (unsigned)(bp >> 32));
    }
    Block *saved = g_block;
    g_block = &b;
    for (;;) {
        bool ran = false;
        for (unsigned t = 0; t < nt; ++t) {
            Fiber &f = b.fibers[t];
            if (f.done || f.waiting) continue;
            b.current = (int)t;
            set_thread(f.tid);
            swapcontext(&b.sched, &f.ctx);
            ran = true;
        }
        // every live fiber is now at the barrier or finished: release the barrier
        int live = 0, total = 0;
        for (auto &f : b.fibers)
            if (!f.done) { ++live; total += f.pred; }
        if (live == 0) break;
        for (auto &f : b.fibers)
            if (!f.done) { f.waiting = false; f.result = total; f.pred = 0; }
        if (!ran) throw std::runtime_error("emulated block made no progress");
    }
    g_block = saved;
}

}  // namespace

int syncthreads_count(int pred) {
    if (!g_block) return pred != 0;   // a block of one thread
    Fiber &f = g_block->fibers[g_block->current];
    f.waiting = true;
    f.pred = pred != 0;
    swapcontext(&f.ctx, &g_block->sched);
    set_thread(f.tid);
    return f.result;
}

void syncthreads() { (void)syncthreads_count(0); }

void launch(const char *name, const Config &cfg, std::function<void()> body) {
    const unsigned nt = cfg.block.x * cfg.block.y * cfg.block.z;
    if (cfg.shmem > sizeof(s) || cfg.shmem > sizeof(cs))
        throw std::runtime_error(std::string("emulated launch needs more shared memory: ") + name);
    if (nt == 0 || cfg.grid.x * cfg.grid.y * cfg.grid.z == 0 || nt > 1024)
        return;   // an invalid configuration launches nothing on the GPU either
    if (std::strcmp(name, "find_string_occurences") == 0) {
        // the real geometry: one block per row, one fiber per thread
        grid_dim = cfg.grid;
        block_dim = cfg.block;
        for (unsigned z = 0; z < cfg.grid.z; ++z)
            for (unsigned y = 0; y < cfg.grid.y; ++y)
                for (unsigned x = 0; x < cfg.grid.x; ++x) {
                    block_idx = uint3{x, y, z};
                    run_block_fibers(cfg, body);
                }
        return;
    }
    // grid-stride kernels: one block of one thread visits every iteration
    grid_dim = dim3(1, 1, 1);
    block_dim = dim3(1, 1, 1);
    block_idx = uint3{0, 0, 0};
    thread_idx = uint3{0, 0, 0};
    body();
}

}  // namespace emu

// CUDA runtime calls of the reference's path, acting on host memory.  The
// device limits reported are those of a current GPU; only the block-size
// arithmetic of the launches reads them (cuda/PSDBSCAN.hcu:977-989).
extern "C" {
cudaError_t CUDARTAPI cudaGetDeviceProperties(struct cudaDeviceProp *prop, int) {
    std::memset(prop, 0, sizeof(*prop));
    std::strcpy(prop->name, "host emulation");
    prop->sharedMemPerBlock = 48 * 1024;
    prop->maxThreadsPerBlock = 1024;
    prop->maxThreadsPerMultiProcessor = 2048;
    prop->maxThreadsDim[0] = 1024;
    prop->maxThreadsDim[1] = 1024;
    prop->maxThreadsDim[2] = 64;
    prop->maxGridSize[0] = 2147483647;
    prop->maxGridSize[1] = 65535;
    prop->maxGridSize[2] = 65535;
    prop->warpSize = 32;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaDeviceSynchronize(void) { return cudaSuccess; }
const char *CUDARTAPI cudaGetErrorString(cudaError_t) { return "no error"; }
cudaError_t CUDARTAPI cudaMalloc(void **p, size_t n) {
    *p = std::malloc(n ? n : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t CUDARTAPI cudaFree(void *p) { std::free(p); return cudaSuccess; }
cudaError_t CUDARTAPI cudaMemcpy(void *d, const void *s, size_t n, enum cudaMemcpyKind) {
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemGetInfo(size_t *free_b, size_t *total_b) {
    *free_b = (size_t)1 << 30;
    *total_b = (size_t)1 << 30;
    return cudaSuccess;
}
}
