// Cluster and block trees on the device (cluster.rs:35-105, block.rs:38-93).
//
// The trees of every body of a batch are built together, level by level:
//   cluster tree: per cluster of the level one CTA takes the bounding box of
//     its points, bisects the box at the midpoint of its longest side
//     (points <= gamma to the first son) and partitions its range of the
//     permutation stably (the sons keep the parent's order, as the
//     reference's push loop does); one single-CTA kernel numbers the sons.
//   block tree: per pair of clusters of the level one thread tests
//     admissibility (min(diam) <= eta * dist) and whether either cluster is a
//     leaf; the pairs that split get four children in the reference's order
//     (son a of the rows with son b of the columns, a outer).  The depth-first
//     order of the leaves (the reference's flattening, block.rs:76-93) comes
//     from leaf counts summed bottom-up and offsets handed top-down.
// Box arithmetic uses explicit round-to-nearest operations without fused
// multiply-adds, the same operation order as the reference, so the trees are
// identical to a sequential FP64 construction.  The host only reads one
// counter per level.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>

#include "tree.cuh"

namespace bem {
namespace {

constexpr int TB = 256;        // threads of the per-cluster box kernel
constexpr int TS = 512;        // threads of the per-cluster partition kernel
constexpr int TSCAN = 1024;    // threads of the single-CTA numbering kernels
constexpr int MAX_DEPTH = 200; // deeper trees are rejected (coincident points)

enum TreeErr { TE_SEPARATE = 1, TE_DEPTH = 2, TE_CAPACITY = 3 };

struct Split {
    double gamma;
    int64_t na;  // points of the first son
    int32_t jmax, go;
};

// Exclusive prefix sum of v over the block; *total receives the block's sum.
// Every thread of the block must call it.
template <int NT>
__device__ __forceinline__ int block_scan(int v, int* sm, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < NT / 32 ? sm[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < NT / 32) sm[lane] = w;
    }
    __syncthreads();
    const int before = warp ? sm[warp - 1] : 0;
    *total = sm[NT / 32 - 1];
    __syncthreads();  // sm is reused by the next call
    return before + x - v;
}

// diam = sqrt(sum (hi - lo)^2) (cluster.rs:84-91)
__device__ __forceinline__ double box_diam(const double* lo, const double* hi) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double e = __dadd_rn(hi[d], -lo[d]);
        s = __dadd_rn(s, __dmul_rn(e, e));
    }
    return __dsqrt_rn(s);
}

// dist = sqrt(sum max(0, a.lo - b.hi)^2 + max(0, b.lo - a.hi)^2) (cluster.rs:94-101)
__device__ __forceinline__ double box_dist(const TreeNode& a, const TreeNode& b) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double t1 = fmax(0.0, __dadd_rn(a.lo[d], -b.hi[d]));
        const double t2 = fmax(0.0, __dadd_rn(b.lo[d], -a.hi[d]));
        s = __dadd_rn(s, __dmul_rn(t1, t1));
        s = __dadd_rn(s, __dmul_rn(t2, t2));
    }
    return __dsqrt_rn(s);
}

// Gathers the collocation points of several bodies (structure of arrays on
// the device, x y z at 0, npad, 2 npad) into one xyz array.
struct BodyGeo {
    const double* x;
    int64_t npad, pt0, n;
};
__global__ void tree_gather_kernel(const BodyGeo* __restrict__ bodies, int nb, int64_t total, double* __restrict__ xyz) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = nb - 1;  // body of point g: the last with pt0 <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bodies[mid].pt0 <= g) lo = mid;
        else hi = mid - 1;
    }
    const BodyGeo b = bodies[lo];
    const int64_t i = g - b.pt0;
    for (int d = 0; d < 3; ++d) xyz[3 * g + d] = b.x[d * b.npad + i];
}

__global__ void tree_init_kernel(int64_t total, int64_t* __restrict__ perm) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < total) perm[g] = g;
}

// One CTA per cluster of the level: bounding box and diameter; for a cluster
// of more than `leaf` points the split plane and the size of the first son.
__global__ void __launch_bounds__(TB) tree_box_kernel(const double* __restrict__ xyz, const int64_t* __restrict__ perm,
                                                      TreeNode* __restrict__ nodes, const int32_t* __restrict__ front,
                                                      int64_t leaf, Split* __restrict__ split, int* __restrict__ err) {
    __shared__ double s_lo[3][TB / 32], s_hi[3][TB / 32];
    __shared__ long long s_cnt[TB / 32];
    __shared__ double s_gamma;
    __shared__ int s_j, s_go;
    const int v = front[blockIdx.x];
    const int64_t b = nodes[v].begin, e = nodes[v].end;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = INFINITY;
        hi[d] = -INFINITY;
    }
    for (int64_t t = b + threadIdx.x; t < e; t += TB) {
        const double* q = xyz + 3 * perm[t];
        for (int d = 0; d < 3; ++d) {
            const double x = q[d];
            lo[d] = fmin(x, lo[d]);
            hi[d] = fmax(x, hi[d]);
        }
    }
    for (int d = 0; d < 3; ++d) {
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
        if (lane == 0) {
            s_lo[d][warp] = lo[d];
            s_hi[d][warp] = hi[d];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int d = 0; d < 3; ++d) {
            for (int w = 1; w < TB / 32; ++w) {
                s_lo[d][0] = fmin(s_lo[d][w], s_lo[d][0]);
                s_hi[d][0] = fmax(s_hi[d][w], s_hi[d][0]);
            }
            lo[d] = s_lo[d][0];
            hi[d] = s_hi[d][0];
            nodes[v].lo[d] = lo[d];
            nodes[v].hi[d] = hi[d];
        }
        nodes[v].diam = box_diam(lo, hi);
        int go = 0, j = 0;
        double gamma = 0.0;
        if (e - b > leaf) {
            if (nodes[v].depth >= MAX_DEPTH) {
                atomicExch(err, TE_DEPTH);
            } else {
                // longest side, the first of equal ones (cluster.rs:50-55)
                double diff = 0.0;
                for (int d = 0; d < 3; ++d) {
                    const double c = __dadd_rn(hi[d], -lo[d]);
                    if (c > diff) {
                        j = d;
                        diff = c;
                    }
                }
                gamma = __dmul_rn(0.5, __dadd_rn(lo[j], hi[j]));
                go = 1;
            }
        }
        s_go = go;
        s_j = j;
        s_gamma = gamma;
    }
    __syncthreads();
    const int go = s_go, j = s_j;
    const double gamma = s_gamma;
    long long cnt = 0;
    if (go)
        for (int64_t t = b + threadIdx.x; t < e; t += TB) cnt += xyz[3 * perm[t] + j] <= gamma;
#pragma unroll
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) s_cnt[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long na = 0;
        for (int w = 0; w < TB / 32; ++w) na += s_cnt[w];
        int ok = go;
        if (go && (na == 0 || na == e - b)) {  // cannot be separated: coincident points
            atomicExch(err, TE_SEPARATE);
            ok = 0;
        }
        split[blockIdx.x] = Split{gamma, (int64_t)na, j, ok};
    }
}

// Single CTA: numbers the sons of the level's splitting clusters (first son
// of the p-th split at base + 2p) and lists them as the next level.
// counters[0]: nodes used; counters[1]: clusters of the next level.
__global__ void __launch_bounds__(TSCAN) tree_number_kernel(TreeNode* __restrict__ nodes,
                                                            const int32_t* __restrict__ front, int nf,
                                                            const Split* __restrict__ split, int32_t* __restrict__ next,
                                                            int* __restrict__ counters, int cap, int* __restrict__ err) {
    __shared__ int sm[TSCAN / 32];
    const int base = counters[0];
    int run = 0;
    for (int c0 = 0; c0 < nf; c0 += TSCAN) {
        const int i = c0 + (int)threadIdx.x;
        const int f = i < nf ? split[i].go : 0;
        int tot;
        const int ex = block_scan<TSCAN>(f, sm, &tot);
        if (f) {
            const int p = run + ex;
            const int a = base + 2 * p;
            if (a + 1 < cap) {
                const int v = front[i];
                const TreeNode pv = nodes[v];
                TreeNode s0{}, s1{};
                s0.begin = pv.begin;
                s0.end = pv.begin + split[i].na;
                s1.begin = s0.end;
                s1.end = pv.end;
                s0.son0 = s0.son1 = s1.son0 = s1.son1 = -1;
                s0.body = s1.body = pv.body;
                s0.depth = s1.depth = pv.depth + 1;
                nodes[a] = s0;
                nodes[a + 1] = s1;
                nodes[v].son0 = a;
                nodes[v].son1 = a + 1;
                next[2 * p] = a;
                next[2 * p + 1] = a + 1;
            } else {
                atomicExch(err, TE_CAPACITY);
            }
        }
        run += tot;
    }
    if (threadIdx.x == 0) {
        counters[0] = base + 2 * run;
        counters[1] = 2 * run;
    }
}

// One CTA per splitting cluster: stable partition of perm[begin .. end) by
// the split plane (first son's points first, each side in the parent's
// order), through `scratch`.
__global__ void __launch_bounds__(TS) tree_partition_kernel(const double* __restrict__ xyz, int64_t* __restrict__ perm,
                                                            int64_t* __restrict__ scratch,
                                                            const TreeNode* __restrict__ nodes,
                                                            const int32_t* __restrict__ front,
                                                            const Split* __restrict__ split) {
    __shared__ int sm[TS / 32];
    const Split sp = split[blockIdx.x];
    if (!sp.go) return;
    const int v = front[blockIdx.x];
    const int64_t b = nodes[v].begin, e = nodes[v].end;
    int64_t run_a = 0, run_b = 0;
    for (int64_t t0 = b; t0 < e; t0 += TS) {
        const int64_t t = t0 + threadIdx.x;
        const bool valid = t < e;
        const int64_t id = valid ? perm[t] : 0;
        const int f = valid && xyz[3 * id + sp.jmax] <= sp.gamma;
        int tot;
        const int ex = block_scan<TS>(f, sm, &tot);
        if (valid) {
            const int64_t pos = f ? run_a + ex : sp.na + run_b + ((int)threadIdx.x - ex);
            scratch[b + pos] = id;
        }
        const int nvalid = (e - t0) < TS ? (int)(e - t0) : TS;
        run_a += tot;
        run_b += nvalid - tot;
    }
    __syncthreads();
    for (int64_t t = b + threadIdx.x; t < e; t += TS) perm[t] = scratch[t];
}

// perm: global point indices -> body-local ones.
__global__ void tree_local_kernel(int64_t total, const int64_t* __restrict__ pt0, int nb, int64_t* __restrict__ perm) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pt0[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    perm[t] -= pt0[lo];
}

// ---- block tree ------------------------------------------------------------
// kind: 0 the pair splits, 1 inadmissible leaf, 3 admissible leaf
__global__ void block_test_kernel(const TreeNode* __restrict__ nodes, const int2* __restrict__ pr, int64_t i0,
                                  int64_t np, double eta, int8_t* __restrict__ kind) {
    const int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i0 + np) return;
    const TreeNode& r = nodes[pr[i].x];
    const TreeNode& c = nodes[pr[i].y];
    const bool adm = fmin(r.diam, c.diam) <= __dmul_rn(eta, box_dist(r, c));
    kind[i] = adm ? 3 : (r.son0 < 0 || c.son0 < 0) ? 1 : 0;
}

// Single CTA: the four children of every splitting pair of the level,
// appended at `next0` (block.rs:38-55: son a of the rows, son b of the
// columns, a outer).  counters[1]: pairs of the next level.
__global__ void __launch_bounds__(TSCAN) block_number_kernel(const TreeNode* __restrict__ nodes,
                                                             int2* __restrict__ pr, const int8_t* __restrict__ kind,
                                                             int32_t* __restrict__ cb, int64_t i0, int np,
                                                             int64_t next0, int64_t cap, int* __restrict__ counters,
                                                             int* __restrict__ err) {
    __shared__ int sm[TSCAN / 32];
    int run = 0;
    for (int c0 = 0; c0 < np; c0 += TSCAN) {
        const int k = c0 + (int)threadIdx.x;
        const int64_t i = i0 + k;
        const int f = k < np && kind[i] == 0;
        int tot;
        const int ex = block_scan<TSCAN>(f, sm, &tot);
        if (f) {
            const int64_t q = next0 + 4 * (int64_t)(run + ex);
            if (q + 3 < cap) {
                const TreeNode& r = nodes[pr[i].x];
                const TreeNode& c = nodes[pr[i].y];
                pr[q + 0] = make_int2(r.son0, c.son0);
                pr[q + 1] = make_int2(r.son0, c.son1);
                pr[q + 2] = make_int2(r.son1, c.son0);
                pr[q + 3] = make_int2(r.son1, c.son1);
                cb[i] = (int32_t)(q - next0);
            } else {
                atomicExch(err, TE_CAPACITY);
            }
        } else if (k < np) {
            cb[i] = -1;
        }
        run += tot;
    }
    if (threadIdx.x == 0) counters[1] = 4 * run;
}

// Leaves below each pair of a level (its children are the next level's
// pairs next0 + cb .. + 3).
__global__ void block_count_kernel(const int8_t* __restrict__ kind, const int32_t* __restrict__ cb, int64_t i0,
                                   int64_t np, int64_t next0, int32_t* __restrict__ cnt) {
    const int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i0 + np) return;
    if (kind[i]) {
        cnt[i] = 1;
    } else {
        const int64_t q = next0 + cb[i];
        cnt[i] = cnt[q] + cnt[q + 1] + cnt[q + 2] + cnt[q + 3];
    }
}

// Root pairs (one per body): first position of each body's leaves.
__global__ void block_root_kernel(int nb, const int32_t* __restrict__ cnt, int32_t* __restrict__ off,
                                  int* __restrict__ total) {
    if (threadIdx.x | blockIdx.x) return;
    int o = 0;
    for (int b = 0; b < nb; ++b) {
        off[b] = o;
        o += cnt[b];
    }
    *total = o;
}

// Hands each pair's first position to its children; a leaf pair writes itself
// at its position (depth-first order).
__global__ void block_place_kernel(const TreeNode* __restrict__ nodes, const int2* __restrict__ pr,
                                   const int8_t* __restrict__ kind, const int32_t* __restrict__ cb,
                                   const int32_t* __restrict__ cnt, int32_t* __restrict__ off, int64_t i0, int64_t np,
                                   int64_t next0, BlockLeaf* __restrict__ out) {
    const int64_t i = i0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i0 + np) return;
    int o = off[i];
    if (kind[i]) {
        out[o] = BlockLeaf{pr[i].x, pr[i].y, kind[i] == 3 ? 1 : 0, nodes[pr[i].x].body};
    } else {
        const int64_t q = next0 + cb[i];
        for (int k = 0; k < 4; ++k) {
            off[q + k] = o;
            o += cnt[q + k];
        }
    }
}

unsigned blocks_for(int64_t n, int t) { return (unsigned)std::max<int64_t>((n + t - 1) / t, 1); }

// Grows a device array to `need` bytes keeping its first `used` bytes.
void grow_keep(Context& c, DevBuf& b, size_t used, size_t need) {
    if (need <= b.bytes) return;
    DevBuf nb;
    nb.ensure(std::max(need, b.bytes + b.bytes / 2));
    if (used) BEM_CUDA(cudaMemcpyAsync(nb.p, b.p, used, cudaMemcpyDeviceToDevice, c.stream));
    c.sync();
    std::swap(nb.p, b.p);
    std::swap(nb.bytes, b.bytes);
}

void tree_error(int e) {
    if (e == TE_SEPARATE || e == TE_DEPTH)
        throw Error(BEM_ERR_BAD_INPUT, "cluster tree: points cannot be separated (coincident collocation points)");
    if (e) throw Error(BEM_ERR_CUDA, "cluster tree: node storage exceeded");
}

// Wall time of a tree stage (it ends with a synchronisation) for the
// library's per-stage profile.
struct TreeTimer {
    Context& c;
    const char* name;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    int64_t l0;
    TreeTimer(Context& ctx, const char* n) : c(ctx), name(n), l0(ctx.launches) {}
    ~TreeTimer() {
        if (c.profiling)
            c.stage_add(name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                        c.launches - l0, 0);
    }
};

// The cluster trees of the points in d_xyz (F.pt0 set by the caller).
void build_forest_dev(Context& c, Forest& F, const DevBuf& d_xyz) {
    TreeTimer timer(c, "cluster_tree");
    const int nb = F.nbodies;
    const int64_t total = F.pt0[(size_t)nb];
    const int cap = (int)std::min<int64_t>(2 * total + 2 * nb + 2, INT32_MAX);
    DevBuf d_nodes, d_scratch, d_front, d_next, d_split, d_cnt, d_pt0;
    d_nodes.ensure(sizeof(TreeNode) * (size_t)cap);
    F.d_perm.ensure(sizeof(int64_t) * (size_t)std::max<int64_t>(total, 1));
    d_scratch.ensure(sizeof(int64_t) * (size_t)std::max<int64_t>(total, 1));
    d_front.ensure(sizeof(int32_t) * (size_t)cap);
    d_next.ensure(sizeof(int32_t) * (size_t)cap);
    d_split.ensure(sizeof(Split) * (size_t)cap);
    d_cnt.ensure(sizeof(int) * 4);
    int64_t* perm = F.d_perm.as<int64_t>();
    // level 0: the roots
    std::vector<TreeNode> roots((size_t)nb);
    std::vector<int32_t> front((size_t)nb);
    for (int b = 0; b < nb; ++b) {
        TreeNode r{};
        r.begin = F.pt0[(size_t)b];
        r.end = F.pt0[(size_t)b + 1];
        r.son0 = r.son1 = -1;
        r.body = b;
        r.depth = 0;
        roots[(size_t)b] = r;
        front[(size_t)b] = b;
    }
    BEM_CUDA(cudaMemcpyAsync(d_nodes.p, roots.data(), sizeof(TreeNode) * nb, cudaMemcpyHostToDevice, c.stream));
    BEM_CUDA(cudaMemcpyAsync(d_front.p, front.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, c.stream));
    int h_cnt[4] = {nb, nb, 0, 0};  // nodes used, clusters of the level, error
    BEM_CUDA(cudaMemcpyAsync(d_cnt.p, h_cnt, sizeof(h_cnt), cudaMemcpyHostToDevice, c.stream));
    int* err = d_cnt.as<int>() + 2;
    if (total) {
        tree_init_kernel<<<blocks_for(total, 256), 256, 0, c.stream>>>(total, perm);
        BEM_CHECK_LAUNCH(&c);
    }
    const double* xyz = d_xyz.as<double>();
    int nf = nb;
    while (nf > 0) {
        tree_box_kernel<<<(unsigned)nf, TB, 0, c.stream>>>(xyz, perm, d_nodes.as<TreeNode>(), d_front.as<int32_t>(),
                                                           F.leaf, d_split.as<Split>(), err);
        BEM_CHECK_LAUNCH(&c);
        tree_number_kernel<<<1, TSCAN, 0, c.stream>>>(d_nodes.as<TreeNode>(), d_front.as<int32_t>(), nf,
                                                      d_split.as<Split>(), d_next.as<int32_t>(), d_cnt.as<int>(), cap,
                                                      err);
        BEM_CHECK_LAUNCH(&c);
        tree_partition_kernel<<<(unsigned)nf, TS, 0, c.stream>>>(xyz, perm, d_scratch.as<int64_t>(),
                                                                 d_nodes.as<TreeNode>(), d_front.as<int32_t>(),
                                                                 d_split.as<Split>());
        BEM_CHECK_LAUNCH(&c);
        BEM_CUDA(cudaMemcpyAsync(h_cnt, d_cnt.p, sizeof(h_cnt), cudaMemcpyDeviceToHost, c.stream));
        c.sync();
        tree_error(h_cnt[2]);
        nf = h_cnt[1];
        std::swap(d_front.p, d_next.p);
    }
    const int nn = h_cnt[0];
    d_pt0.ensure(sizeof(int64_t) * F.pt0.size());
    BEM_CUDA(cudaMemcpyAsync(d_pt0.p, F.pt0.data(), sizeof(int64_t) * F.pt0.size(), cudaMemcpyHostToDevice, c.stream));
    if (total) {
        tree_local_kernel<<<blocks_for(total, 256), 256, 0, c.stream>>>(total, d_pt0.as<int64_t>(), nb, perm);
        BEM_CHECK_LAUNCH(&c);
    }
    F.nodes.resize((size_t)nn);
    F.perm.resize((size_t)total);
    BEM_CUDA(cudaMemcpyAsync(F.nodes.data(), d_nodes.p, sizeof(TreeNode) * nn, cudaMemcpyDeviceToHost, c.stream));
    if (total)
        BEM_CUDA(cudaMemcpyAsync(F.perm.data(), perm, sizeof(int64_t) * total, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    // node ranges are in the global numbering of the concatenated points:
    // make them body-local, and list the leaves depth-first (first son first)
    for (TreeNode& v : F.nodes) {
        v.begin -= F.pt0[(size_t)v.body];
        v.end -= F.pt0[(size_t)v.body];
    }
    F.leaves.clear();
    F.leaf0.assign(1, 0);
    std::vector<int32_t> stack;
    for (int b = 0; b < nb; ++b) {
        stack.assign(1, b);
        while (!stack.empty()) {
            const int v = stack.back();
            stack.pop_back();
            const TreeNode& x = F.nodes[(size_t)v];
            if (x.son0 < 0) {
                F.leaves.push_back(v);
            } else {
                stack.push_back(x.son1);
                stack.push_back(x.son0);
            }
        }
        F.leaf0.push_back((int32_t)F.leaves.size());
    }
}

}  // namespace

double node_distance(const TreeNode& a, const TreeNode& b) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double t1 = std::fmax(0.0, a.lo[d] - b.hi[d]);
        const double t2 = std::fmax(0.0, b.lo[d] - a.hi[d]);
        s += t1 * t1;
        s += t2 * t2;
    }
    return std::sqrt(s);
}

std::shared_ptr<Forest> build_forest(Context& c, int nb, const double* const* pts, const int64_t* npts,
                                     int64_t stride, int64_t leaf) {
    require(nb >= 1 && stride >= 3 && leaf >= 1, "cluster tree: bad arguments");
    auto F = std::make_shared<Forest>();
    F->nbodies = nb;
    F->leaf = leaf;
    F->pt0.assign(1, 0);
    for (int b = 0; b < nb; ++b) {
        require(npts[b] >= 0, "cluster tree: negative point count");
        F->pt0.push_back(F->pt0.back() + npts[b]);
    }
    const int64_t total = F->pt0.back();
    std::vector<double> h((size_t)(3 * std::max<int64_t>(total, 1)));
    for (int b = 0; b < nb; ++b)
        for (int64_t i = 0; i < npts[b]; ++i)
            for (int d = 0; d < 3; ++d) h[(size_t)(3 * (F->pt0[(size_t)b] + i) + d)] = pts[b][stride * i + d];
    DevBuf d_xyz;
    d_xyz.ensure(sizeof(double) * h.size());
    BEM_CUDA(cudaMemcpyAsync(d_xyz.p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, c.stream));
    build_forest_dev(c, *F, d_xyz);
    return F;
}

std::shared_ptr<Forest> build_forest(Context& c, const std::vector<const Problem*>& bodies, int64_t leaf) {
    const int nb = (int)bodies.size();
    require(nb >= 1 && leaf >= 1, "cluster tree: bad arguments");
    auto F = std::make_shared<Forest>();
    F->nbodies = nb;
    F->leaf = leaf;
    F->pt0.assign(1, 0);
    std::vector<BodyGeo> g((size_t)nb);
    for (int b = 0; b < nb; ++b) {
        const Problem& p = *bodies[(size_t)b];
        g[(size_t)b] = BodyGeo{p.geo.buf.as<double>() + GX * p.geo.npad, p.geo.npad, F->pt0.back(), p.n};
        F->pt0.push_back(F->pt0.back() + p.n);
    }
    const int64_t total = F->pt0.back();
    DevBuf d_xyz, d_g;
    d_xyz.ensure(sizeof(double) * (size_t)(3 * std::max<int64_t>(total, 1)));
    d_g.ensure(sizeof(BodyGeo) * (size_t)nb);
    BEM_CUDA(cudaMemcpyAsync(d_g.p, g.data(), sizeof(BodyGeo) * nb, cudaMemcpyHostToDevice, c.stream));
    if (total) {
        tree_gather_kernel<<<blocks_for(total, 256), 256, 0, c.stream>>>(d_g.as<BodyGeo>(), nb, total,
                                                                         d_xyz.as<double>());
        BEM_CHECK_LAUNCH(&c);
    }
    build_forest_dev(c, *F, d_xyz);
    return F;
}

std::vector<BlockLeaf> forest_block_leaves(Context& c, const Forest& F, double eta) {
    TreeTimer timer(c, "block_tree");
    const int nb = F.nbodies;
    DevBuf d_nodes, d_pr, d_kind, d_cb, d_cnt, d_off, d_ctr, d_out;
    // the block tree reads boxes, diameters and sons only
    d_nodes.ensure(sizeof(TreeNode) * F.nodes.size());
    BEM_CUDA(cudaMemcpyAsync(d_nodes.p, F.nodes.data(), sizeof(TreeNode) * F.nodes.size(), cudaMemcpyHostToDevice,
                             c.stream));
    size_t cap = std::max<size_t>(1024, (size_t)nb * 64);
    d_pr.ensure(sizeof(int2) * cap);
    d_kind.ensure(cap);
    d_cb.ensure(sizeof(int32_t) * cap);
    d_ctr.ensure(sizeof(int) * 4);
    std::vector<int2> roots((size_t)nb);
    for (int b = 0; b < nb; ++b) roots[(size_t)b] = make_int2(b, b);
    BEM_CUDA(cudaMemcpyAsync(d_pr.p, roots.data(), sizeof(int2) * nb, cudaMemcpyHostToDevice, c.stream));
    int h_ctr[4] = {0, 0, 0, 0};
    BEM_CUDA(cudaMemcpyAsync(d_ctr.p, h_ctr, sizeof(h_ctr), cudaMemcpyHostToDevice, c.stream));
    int* err = d_ctr.as<int>() + 2;
    std::vector<int64_t> lvl(1, 0);  // first pair of each level
    int64_t i0 = 0, np = nb;
    while (np > 0) {
        const int64_t next0 = i0 + np;
        const size_t need = (size_t)(next0 + 4 * np);
        if (need > cap) {
            const size_t ncap = std::max(need, cap + cap / 2);
            grow_keep(c, d_pr, sizeof(int2) * (size_t)next0, sizeof(int2) * ncap);
            grow_keep(c, d_kind, (size_t)next0, ncap);
            grow_keep(c, d_cb, sizeof(int32_t) * (size_t)next0, sizeof(int32_t) * ncap);
            cap = ncap;
        }
        block_test_kernel<<<blocks_for(np, 256), 256, 0, c.stream>>>(d_nodes.as<TreeNode>(), d_pr.as<int2>(), i0, np,
                                                                     eta, d_kind.as<int8_t>());
        BEM_CHECK_LAUNCH(&c);
        require(np < INT32_MAX, "block tree: level too large", BEM_ERR_CUDA);
        block_number_kernel<<<1, TSCAN, 0, c.stream>>>(d_nodes.as<TreeNode>(), d_pr.as<int2>(), d_kind.as<int8_t>(),
                                                       d_cb.as<int32_t>(), i0, (int)np, next0, (int64_t)cap,
                                                       d_ctr.as<int>(), err);
        BEM_CHECK_LAUNCH(&c);
        BEM_CUDA(cudaMemcpyAsync(h_ctr, d_ctr.p, sizeof(h_ctr), cudaMemcpyDeviceToHost, c.stream));
        c.sync();
        tree_error(h_ctr[2]);
        i0 = next0;
        np = h_ctr[1];
        lvl.push_back(i0);
    }
    const int64_t npairs = i0;
    const int nl = (int)lvl.size() - 1;  // levels: [lvl[L], lvl[L + 1])
    d_cnt.ensure(sizeof(int32_t) * (size_t)npairs);
    d_off.ensure(sizeof(int32_t) * (size_t)npairs);
    for (int L = nl - 1; L >= 0; --L) {
        const int64_t a = lvl[(size_t)L], m = lvl[(size_t)L + 1] - a;
        block_count_kernel<<<blocks_for(m, 256), 256, 0, c.stream>>>(d_kind.as<int8_t>(), d_cb.as<int32_t>(), a, m,
                                                                     lvl[(size_t)L + 1], d_cnt.as<int32_t>());
        BEM_CHECK_LAUNCH(&c);
    }
    block_root_kernel<<<1, 1, 0, c.stream>>>(nb, d_cnt.as<int32_t>(), d_off.as<int32_t>(), d_ctr.as<int>() + 3);
    BEM_CHECK_LAUNCH(&c);
    BEM_CUDA(cudaMemcpyAsync(h_ctr, d_ctr.p, sizeof(h_ctr), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    const int nleaf = h_ctr[3];
    d_out.ensure(sizeof(BlockLeaf) * (size_t)std::max(nleaf, 1));
    for (int L = 0; L < nl; ++L) {
        const int64_t a = lvl[(size_t)L], m = lvl[(size_t)L + 1] - a;
        block_place_kernel<<<blocks_for(m, 256), 256, 0, c.stream>>>(
            d_nodes.as<TreeNode>(), d_pr.as<int2>(), d_kind.as<int8_t>(), d_cb.as<int32_t>(), d_cnt.as<int32_t>(),
            d_off.as<int32_t>(), a, m, lvl[(size_t)L + 1], d_out.as<BlockLeaf>());
        BEM_CHECK_LAUNCH(&c);
    }
    std::vector<BlockLeaf> out((size_t)nleaf);
    BEM_CUDA(cudaMemcpyAsync(out.data(), d_out.p, sizeof(BlockLeaf) * nleaf, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    return out;
}

}  // namespace bem

// ---------------------------------------------------------------------------
// C ABI: Cluster::new_from (cluster.rs:23-31) and BlockList::new_from over a
// BlockTree (block.rs:20-28, :76-93) for several point sets.
extern "C" BEM_API bem_status bem_cluster_tree(bem_ctx* ctx, int nsets, const int64_t* npts, const double* pts,
                                               int64_t stride, int64_t leaf, double eta, int64_t* perm,
                                               int64_t* leaves, int64_t leaf_cap, int64_t* nleaves, int64_t* blocks,
                                               int64_t block_cap, int64_t* nblocks, double* root_diam) {
    if (!ctx || nsets < 1 || !npts || !perm || !nleaves || !nblocks) return BEM_ERR_BAD_INPUT;
    try {
        bem::Context& c = ctx->c;
        BEM_CUDA(cudaSetDevice(c.device));
        std::vector<const double*> ptr((size_t)nsets);
        int64_t off = 0;
        for (int s = 0; s < nsets; ++s) {
            bem::require(npts[s] >= 0, "cluster tree: negative point count");
            ptr[(size_t)s] = pts + stride * off;
            off += npts[s];
        }
        bem::require(off == 0 || pts, "cluster tree: no points");
        auto F = bem::build_forest(c, nsets, ptr.data(), npts, stride, leaf);
        std::memcpy(perm, F->perm.data(), sizeof(int64_t) * F->perm.size());
        if (root_diam)
            for (int s = 0; s < nsets; ++s) root_diam[s] = F->root((int)s).diam;
        *nleaves = (int64_t)F->leaves.size();
        std::vector<bem::BlockLeaf> bl;
        if (eta >= 0) bl = bem::forest_block_leaves(c, *F, eta);
        *nblocks = (int64_t)bl.size();
        bem::require(*nleaves <= leaf_cap && (*nblocks <= block_cap || eta < 0),
                     "cluster tree: output arrays too small (counts returned)");
        bem::require((leaves || !*nleaves) && (blocks || !*nblocks), "cluster tree: null output array");
        for (size_t l = 0; l < F->leaves.size(); ++l) {
            const bem::TreeNode& v = F->nodes[(size_t)F->leaves[l]];
            leaves[3 * l] = v.body;
            leaves[3 * l + 1] = v.begin;
            leaves[3 * l + 2] = v.end;
        }
        for (size_t b = 0; b < bl.size(); ++b) {
            const bem::TreeNode& r = F->nodes[(size_t)bl[b].r];
            const bem::TreeNode& q = F->nodes[(size_t)bl[b].c];
            int64_t* o = blocks + 6 * b;
            o[0] = bl[b].body;
            o[1] = r.begin;
            o[2] = r.end;
            o[3] = q.begin;
            o[4] = q.end;
            o[5] = bl[b].adm;
        }
        return BEM_OK;
    } catch (const bem::Error& e) {
        ctx->c.last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        ctx->c.last_error = e.what();
        return BEM_ERR_CUDA;
    }
}
