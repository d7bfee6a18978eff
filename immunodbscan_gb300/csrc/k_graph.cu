// k_graph.cu -- neighbour graph, core points, cluster growth and labels
// (rules S5-S7).
//
// Reference counterparts:
//  core counts (S5)  cuda/PSDBSCAN.hcu:1099 (count starts at copies), :824-826 /
//                    :648-650 (each neighbour pair adds the other side's copies),
//                    :1180 (core = count >= minPts)
//  growth (S6)       cuda/PSDBSCAN.hcu:866-926: core-core neighbours are merged by
//                    union_a_and_b (:76-107, link towards the smaller index), a
//                    non-core neighbour is claimed by the first core to win an
//                    atomicCAS (:113-122)
//  labels (S7)       cuda/PSDBSCAN.hcu:1263-1294 (+ tree_reduction_kernel :129-149)
//  tree depths       cuda/PSDBSCAN.hcu:154-177, 1020-1040
//
// Here the neighbour pairs found by the distance kernel form an edge list.
// Counts are accumulated per edge; core-core edges are merged by unions that
// hook the larger root under the smaller one with atomicCAS while find()
// halves paths, so every component's root is its minimum core index, as in the
// reference.  In the same pass every core-to-non-core edge offers its core end
// to the non-core end with atomicMin, so a non-core unique joins the cluster
// of its minimum-index core neighbour (deterministic; one of the outcomes the
// reference's race allows).  Labels are 1 + the rank of the root among the
// repertoire's core roots, found with one exclusive scan over root flags.
#include "idb_internal.cuh"

namespace idb {

namespace {

constexpr int kThreads = 256;

inline int grid_for(uint64_t n, int threads = kThreads) {
    uint64_t g = (n + threads - 1) / threads;
    uint64_t cap = (uint64_t)sm_count() * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

__device__ __forceinline__ uint32_t edge_slots(const Counters *ctr, uint64_t cap) {
    const uint64_t r = ctr->edge_reserved;
    return (uint32_t)(r < cap ? r : cap);
}

__global__ void k_graph_init(const Counters *__restrict__ ctr, const uint32_t *__restrict__ ucopies,
                             uint32_t *__restrict__ cnt, uint32_t *__restrict__ parent,
                             uint32_t *__restrict__ bmin) {
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        cnt[u] = ucopies[u];
        parent[u] = u;
        bmin[u] = kNone;
    }
}

// count pass: copies-weighted neighbour counts (S5)
__global__ void k_count(const Counters *__restrict__ ctr, uint64_t cap, const uint2 *__restrict__ edges,
                        const uint32_t *__restrict__ ucopies, uint32_t *__restrict__ cnt) {
    const uint32_t ne = edge_slots(ctr, cap);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
        const uint2 ed = edges[e];
        if (ed.x == kNone) continue;
        atomicAdd(&cnt[ed.x], ucopies[ed.y]);
        atomicAdd(&cnt[ed.y], ucopies[ed.x]);
    }
}

__global__ void k_core(const Counters *__restrict__ ctr0, Counters *ctr, const uint32_t *__restrict__ cnt,
                       uint32_t min_pts, uint32_t *__restrict__ ucore) {
    const uint32_t nu = ctr0->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t local = 0;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        const uint32_t c = cnt[u] >= min_pts;
        ucore[u] = c;
        local += c;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) local += __shfl_xor_sync(0xFFFFFFFFu, local, d);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(&ctr->n_cores, local);
}

__device__ __forceinline__ uint32_t uf_find(uint32_t *p, uint32_t x) {
    volatile uint32_t *vp = p;
    while (true) {   // parent[y] <= y always, so x strictly decreases: terminates
        const uint32_t px = vp[x];
        if (px == x) return x;
        const uint32_t ppx = vp[px];
        if (ppx == px) return px;
        vp[x] = ppx;           // path halving
        x = ppx;
    }
}

// Core-core edges are merged (S6); an edge with one core end offers the core
// to its non-core end, which keeps the minimum (the border rule).
__global__ void k_union(Counters *ctr, uint64_t cap, const uint2 *__restrict__ edges,
                        const uint32_t *__restrict__ ucore, uint32_t *parent,
                        uint32_t *__restrict__ bmin) {
    const uint32_t ne = edge_slots(ctr, cap);
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t n_cc = 0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
        const uint2 ed = edges[e];
        if (ed.x == kNone) continue;
        const uint32_t cx = ucore[ed.x], cy = ucore[ed.y];
        if (cx != cy) { atomicMin(&bmin[cx ? ed.y : ed.x], cx ? ed.x : ed.y); continue; }
        if (!cx) continue;
        ++n_cc;
        uint32_t a = ed.x, b = ed.y;
        uint32_t it = 0;
        for (; it < kSpinCap; ++it) {
            uint32_t ra = uf_find(parent, a), rb = uf_find(parent, b);
            if (ra == rb) break;
            if (ra < rb) { const uint32_t t = ra; ra = rb; rb = t; }
            // hook the larger root under the smaller one
            if (atomicCAS(&parent[ra], ra, rb) == ra) break;
            a = ra;
            b = rb;
        }
        if (it == kSpinCap) atomicOr(&ctr->error, kErrUnionStall);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) n_cc += __shfl_xor_sync(0xFFFFFFFFu, n_cc, d);
    if ((threadIdx.x & 31) == 0 && n_cc) atomicAdd(&ctr->n_core_edges, n_cc);
}

// depth of every row in the union-find forest before compression (diagnostic)
__global__ void k_depth(uint32_t N, const uint32_t *__restrict__ row2uid, const uint32_t *__restrict__ urow,
                        const uint32_t *__restrict__ ucore, const uint32_t *__restrict__ bmin,
                        const uint32_t *parent, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[kDepthMax + 1];
    for (int k = threadIdx.x; k <= kDepthMax; k += blockDim.x) h[k] = 0;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
        const uint32_t u = row2uid[i];
        uint32_t depth = urow[u] != i;                  // duplicate -> representative
        uint32_t x = u;
        if (!ucore[u]) {
            if (bmin[u] == kNone) x = kNone;
            else { x = bmin[u]; ++depth; }
        }
        if (x != kNone)
            while (depth < kDepthMax) {
                const uint32_t px = parent[x];
                if (px == x) break;
                x = px;
                ++depth;
            }
        atomicAdd(&h[min(depth, (uint32_t)kDepthMax)], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k <= kDepthMax; k += blockDim.x)
        if (h[k]) atomicAdd(&hist[k], h[k]);
}

// Full compression: parent[u] = root of u for every core u.  The walk to the
// root only reads: with path halving here, a halving step computed from a stale
// parent could land after another thread's final root write and leave that
// node pointing at an inner ancestor.  Each thread writes only its own node,
// and the roots no longer change, so every write is final.
__global__ void k_compress(const Counters *__restrict__ ctr, const uint32_t *__restrict__ ucore,
                           uint32_t *parent, uint32_t *__restrict__ rootflag) {
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    volatile uint32_t *vp = parent;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        uint32_t r = u;
        if (ucore[u]) {
            uint32_t pr = vp[r];
            while (pr != r) {   // parent[y] <= y: strictly decreasing, terminates
                r = pr;
                pr = vp[r];
            }
            parent[u] = r;
        }
        rootflag[u] = ucore[u] && r == u;
    }
}

__global__ void k_labels(const Counters *__restrict__ ctr, const uint32_t *__restrict__ ucore,
                         const uint32_t *__restrict__ parent, const uint32_t *__restrict__ bmin,
                         const uint32_t *__restrict__ rank, const uint32_t *__restrict__ urep,
                         const uint32_t *__restrict__ uid_first, uint32_t *__restrict__ ulabel) {
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) {
        uint32_t root = kNone;
        if (ucore[u]) root = parent[u];
        else if (bmin[u] != kNone) root = parent[bmin[u]];
        uint32_t lab = 0;
        if (root != kNone) lab = rank[root] - rank[uid_first[urep[u]]] + 1;
        ulabel[u] = lab;
    }
}

// Row outputs.  `what` selects them (kOutClone / kOutCore / kOutCopies): the
// copies are final once the uniques exist and the core flags once the counts
// are, so a call can write (and copy out) those two before the labels.
__global__ void k_rows_out(uint32_t N, uint32_t min_pts, const uint32_t *__restrict__ row2uid,
                           const uint32_t *__restrict__ urow, const uint32_t *__restrict__ ucopies,
                           const uint32_t *__restrict__ ucore, const uint32_t *__restrict__ ulabel,
                           uint32_t *__restrict__ clone_id, int32_t *__restrict__ core,
                           uint32_t *__restrict__ copies, Counters *ctr, uint32_t what) {
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t noise = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
        const uint32_t u = row2uid[i];
        const bool rep = urow[u] == i;
        if (what & kOutCopies) copies[i] = rep ? ucopies[u] : 0u;
        // a duplicate keeps count 0 and is core only for minPts == 0
        if (what & kOutCore) core[i] = rep ? (int32_t)ucore[u] : (int32_t)(min_pts == 0);
        if (what & kOutClone) {
            const uint32_t lab = ulabel[u];
            clone_id[i] = lab;
            noise += lab == 0;
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) noise += __shfl_xor_sync(0xFFFFFFFFu, noise, d);
    if ((threadIdx.x & 31) == 0 && noise) atomicAdd(&ctr->n_noise_rows, noise);
}

__global__ void k_uniques_out(const Counters *__restrict__ ctr, const uint32_t *__restrict__ urow,
                              uint32_t *__restrict__ out) {
    const uint32_t nu = ctr->n_uniques;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nu; u += stride) out[u] = urow[u];
}

}  // namespace

void launch_graph(const Plan &P, const Buffers &B, bool trees, cudaStream_t s, cudaEvent_t core_out) {
    const uint64_t ecap = P.cap_edges;
    const int gu = grid_for(P.N);
    k_graph_init<<<grid_wave(k_graph_init, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ucopies, B.cnt, B.parent, B.bmin);
    k_count<<<grid_wave(k_count, ecap, kThreads), kThreads, 0, s>>>(B.ctr, ecap, B.edges, B.ucopies, B.cnt);
    k_core<<<grid_wave(k_core, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ctr, B.cnt, P.min_pts, B.ucore);
    if (core_out) {   // the row core flags now, and an event for their copy
        launch_outputs(P, B, s, kOutCore);
        cudaEventRecordWithFlags(core_out, s, cudaEventRecordExternal);
    }
    // unions of core-core edges; each non-core unique keeps its minimum core neighbour
    k_union<<<grid_wave(k_union, ecap, kThreads), kThreads, 0, s>>>(B.ctr, ecap, B.edges, B.ucore, B.parent, B.bmin);
    if (trees) {
        cudaMemsetAsync(B.depth_hist, 0, sizeof(uint32_t) * (kDepthMax + 1), s);
        k_depth<<<gu, kThreads, 0, s>>>(P.N, B.row2uid, B.urow, B.ucore, B.bmin, B.parent,
                                         B.depth_hist);
    }
    cudaMemsetAsync(B.rootflag, 0, sizeof(uint32_t) * ((size_t)P.N + 1), s);
    k_compress<<<grid_wave(k_compress, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ucore, B.parent, B.rootflag);
    scan_u32(B.rootflag, B.rootflag, P.N + 1, nullptr, &B.ctr->n_clusters, B.scan_part,
             B.scan_part_cap, s);
    k_labels<<<grid_wave(k_labels, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ucore, B.parent, B.bmin, B.rootflag, B.urep,
                                      B.uid_first, B.cnt);
}

// Streamed mode: counts from a first distance sweep, core flags, then a second
// sweep that merges core-core pairs and keeps every non-core unique's minimum
// core neighbour; depths, compression and labels as above.  The sweep-local
// statistics are cleared between the sweeps so that they count one sweep.
void launch_streamed_sweeps(const Plan &P, const Buffers &B, cudaStream_t s) {
    k_graph_init<<<grid_wave(k_graph_init, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ucopies, B.cnt, B.parent, B.bmin);
    launch_distance(P, B, 0, s, kSinkCount);
    k_core<<<grid_wave(k_core, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ctr, B.cnt, P.min_pts, B.ucore);
    cudaMemsetAsync(&B.ctr->pairs_evaluated, 0, sizeof(B.ctr->pairs_evaluated), s);
    cudaMemsetAsync(&B.ctr->n_edges, 0, sizeof(B.ctr->n_edges), s);
    cudaMemsetAsync(&B.ctr->edge_reserved, 0, sizeof(B.ctr->edge_reserved), s);
    cudaMemsetAsync(&B.ctr->lev_columns, 0, sizeof(B.ctr->lev_columns), s);
    launch_distance(P, B, 0, s, kSinkGrow);
}

void launch_streamed_labels(const Plan &P, const Buffers &B, bool trees, cudaStream_t s) {
    if (trees) {
        cudaMemsetAsync(B.depth_hist, 0, sizeof(uint32_t) * (kDepthMax + 1), s);
        k_depth<<<grid_for(P.N), kThreads, 0, s>>>(P.N, B.row2uid, B.urow, B.ucore, B.bmin, B.parent,
                                                   B.depth_hist);
    }
    cudaMemsetAsync(B.rootflag, 0, sizeof(uint32_t) * ((size_t)P.N + 1), s);
    k_compress<<<grid_wave(k_compress, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ucore, B.parent, B.rootflag);
    scan_u32(B.rootflag, B.rootflag, P.N + 1, nullptr, &B.ctr->n_clusters, B.scan_part,
             B.scan_part_cap, s);
    k_labels<<<grid_wave(k_labels, P.N, kThreads), kThreads, 0, s>>>(B.ctr, B.ucore, B.parent, B.bmin, B.rootflag, B.urep,
                                      B.uid_first, B.cnt);
}

void launch_outputs(const Plan &P, const Buffers &B, cudaStream_t s, uint32_t what) {
    const int gu = grid_for(P.N);
    k_rows_out<<<grid_wave(k_rows_out, P.N, kThreads), kThreads, 0, s>>>(P.N, P.min_pts, B.row2uid, B.urow, B.ucopies, B.ucore,
                                        B.cnt, B.clone_id, B.core, B.copies, B.ctr, what);
    if (B.uniques && (what & kOutClone)) k_uniques_out<<<gu, kThreads, 0, s>>>(B.ctr, B.urow, B.uniques);
}

}  // namespace idb
