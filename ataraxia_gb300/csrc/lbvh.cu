// GPU construction of the linear BVH over the spheres (no counterpart in the
// reference, whose traceRay is an O(N) loop, Renderer.cu:256-279).
//
//   1. bounds of the sphere centres (block reduction + one atomic per block)
//   2. 30-bit Morton code per sphere: centre normalised to the bounds,
//      10 bits per axis, bits interleaved x-y-z
//   3. stable LSD radix sort of (code, sphere index), 8 bits per pass; the
//      input is in index order, so equal codes stay in index order
//   4. Karras' binary radix tree ("Maximizing Parallelism in the Construction
//      of BVHs, Octrees, and k-d Trees", HPG 2012): one thread per internal
//      node finds its range and split from the longest-common-prefix function
//      over (code, sorted position), which makes every key distinct
//   5. bottom-up boxes: each leaf thread climbs, the second arrival at a node
//      forms the union of its children's boxes
//   6. 4-wide nodes for traversal (the four grandchildren's boxes in two
//      lines, subtrees of at most leaf_size spheres collapsed into leaf
//      clusters)
#include <cstdint>

#include "lbvh.h"
#include "device_math.cuh"

namespace atx {
namespace {

constexpr int kT = 256;
constexpr int kTile = 4096;   // keys per sort block
constexpr int kWarps = kT / 32;

__device__ __forceinline__ unsigned f2ord(float f)
{
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// bounds[0..2] = ordered min, [3..5] = ordered max
__global__ void k_bounds(const float4* sph, uint32_t n, unsigned* bounds)
{
    float lo[3] = {kFltMax, kFltMax, kFltMax}, hi[3] = {-kFltMax, -kFltMax, -kFltMax};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 s = sph[i];
        lo[0] = fminf(lo[0], s.x); lo[1] = fminf(lo[1], s.y); lo[2] = fminf(lo[2], s.z);
        hi[0] = fmaxf(hi[0], s.x); hi[1] = fmaxf(hi[1], s.y); hi[2] = fmaxf(hi[2], s.z);
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) {
            atomicMin(&bounds[k], f2ord(lo[k]));
            atomicMax(&bounds[3 + k], f2ord(hi[k]));
        }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_morton(const float4* sph, uint32_t n, const unsigned* bounds, uint32_t* codes, uint32_t* idx)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 s = sph[i];
    const float p[3] = {s.x, s.y, s.z};
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        const float lo = ord2f(bounds[k]), hi = ord2f(bounds[3 + k]);
        const float ext = hi - lo;
        float u = ext > 0.0f ? (p[k] - lo) / ext : 0.0f;
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        q[k] = (uint32_t)fminf(u * 1024.0f, 1023.0f);
    }
    codes[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    idx[i] = i;
}

// counts[digit * nblocks + block]
__global__ void k_sort_hist(const uint32_t* keys, uint32_t n, int shift, uint32_t* counts)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t start = blockIdx.x * kTile;
    const uint32_t end = min(n, start + kTile);
    for (uint32_t i = start + threadIdx.x; i < end; i += kT) atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
    __syncthreads();
    counts[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of counts in place, one block.
__global__ void k_sort_scan(uint32_t* counts, uint32_t m)
{
    __shared__ uint32_t carry;
    __shared__ uint32_t warp_sums[kWarps];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < m; base += kT) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < m ? counts[i] : 0u;
        uint32_t x = v;
        const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= (uint32_t)off) x += y;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        uint32_t wpre = 0;
        for (uint32_t k = 0; k < w; ++k) wpre += warp_sums[k];
        const uint32_t c = carry;
        if (i < m) counts[i] = c + wpre + x - v;
        __syncthreads();
        if (threadIdx.x == kT - 1) carry = c + wpre + x;
        __syncthreads();
    }
}

// Stable scatter: chunks of kT keys in order; within a chunk the rank of a key
// among equal digits is (keys of that digit in earlier warps) + (earlier lanes
// of its warp with that digit).
__global__ void k_sort_scatter(const uint32_t* keys, const uint32_t* vals, uint32_t n, int shift,
                               const uint32_t* offsets, uint32_t* keys_out, uint32_t* vals_out)
{
    __shared__ uint32_t base[256];
    __shared__ uint32_t wh[kWarps][256];
    __shared__ uint32_t total[256];
    base[threadIdx.x] = offsets[threadIdx.x * gridDim.x + blockIdx.x];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t start = blockIdx.x * kTile;
    const uint32_t end = min(n, start + kTile);
    for (uint32_t c0 = start; c0 < end; c0 += kT) {
        for (int k = 0; k < kWarps; ++k) wh[k][threadIdx.x] = 0;
        __syncthreads();
        const uint32_t i = c0 + threadIdx.x;
        const bool valid = i < end;
        const uint32_t key = valid ? keys[i] : 0u;
        const uint32_t dig = valid ? ((key >> shift) & 0xffu) : 256u + lane;  // invalid lanes never match
        const unsigned peers = __match_any_sync(0xffffffffu, dig);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wh[w][dig] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = 0;
            for (int k = 0; k < kWarps; ++k) {
                const uint32_t t = wh[k][threadIdx.x];
                wh[k][threadIdx.x] = run;
                run += t;
            }
            total[threadIdx.x] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = base[dig] + wh[w][dig] + rank;
            keys_out[pos] = key;
            vals_out[pos] = vals[i];
        }
        __syncthreads();
        base[threadIdx.x] += total[threadIdx.x];
        __syncthreads();
    }
}

// Longest common prefix of the keys (code, position) at sorted positions i, j.
__device__ __forceinline__ int delta(const uint32_t* codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = codes[i], b = codes[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void k_tree(const uint32_t* codes, int n, float4* node_ctr, float4* node_half, uint2* range,
                       uint32_t* parent)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(codes, n, i, i - d);
    int lmax = 2;
    while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(codes, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + (d < 0 ? -1 : 0);
    const int lo = min(i, j), hi = max(i, j);
    const uint32_t left = (lo == gamma) ? (uint32_t)(n - 1 + gamma) : (uint32_t)gamma;
    const uint32_t right = (hi == gamma + 1) ? (uint32_t)(n - 1 + gamma + 1) : (uint32_t)(gamma + 1);
    node_ctr[i].w = __uint_as_float(left);
    node_half[i].w = __uint_as_float(right);
    range[i] = make_uint2((uint32_t)lo, (uint32_t)hi);
    parent[left] = (uint32_t)i;
    parent[right] = (uint32_t)i;
}

__global__ void k_gather_leaves(const float4* sph, const float* radius, const uint32_t* order, int n,
                                float4* leaf_sph, uint32_t* leaf_id, float4* node_ctr, float4* node_half)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t id = order[k];
    const float4 s = sph[id];
    const float r = fabsf(radius[id]);
    leaf_sph[k] = s;
    leaf_id[k] = id;
    node_ctr[n - 1 + k] = make_float4(s.x, s.y, s.z, 0.0f);
    node_half[n - 1 + k] = make_float4(r, r, r, 0.0f);
}

__global__ void k_refit(int n, float4* node_ctr, float4* node_half, const uint32_t* parent, uint32_t* visits)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || n < 2) return;
    uint32_t node = (uint32_t)(n - 1 + k);
    for (int depth = 0; depth < 128; ++depth) {
        if (node == 0u) break;
        const uint32_t p = parent[node];
        __threadfence();
        if (atomicAdd(&visits[p], 1u) == 0u) break;  // first arrival: the sibling finishes
        __threadfence();
        const float4 pc = node_ctr[p], ph = node_half[p];
        const uint32_t l = __float_as_uint(pc.w), r = __float_as_uint(ph.w);
        const float4 c0 = __ldcg(&node_ctr[l]), h0 = __ldcg(&node_half[l]);
        const float4 c1 = __ldcg(&node_ctr[r]), h1 = __ldcg(&node_half[r]);
        const float lx = fminf(c0.x - h0.x, c1.x - h1.x), hx = fmaxf(c0.x + h0.x, c1.x + h1.x);
        const float ly = fminf(c0.y - h0.y, c1.y - h1.y), hy = fmaxf(c0.y + h0.y, c1.y + h1.y);
        const float lz = fminf(c0.z - h0.z, c1.z - h1.z), hz = fmaxf(c0.z + h0.z, c1.z + h1.z);
        const float cx = 0.5f * (lx + hx), cy = 0.5f * (ly + hy), cz = 0.5f * (lz + hz);
        // round the half extent up so the stored box contains both children
        const float ex = fmaxf(hx - cx, cx - lx), ey = fmaxf(hy - cy, cy - ly), ez = fmaxf(hz - cz, cz - lz);
        const float slack = 1e-6f * (fabsf(cx) + fabsf(cy) + fabsf(cz) + ex + ey + ez) + 1e-30f;
        __stcg(&node_ctr[p], make_float4(cx, cy, cz, pc.w));
        __stcg(&node_half[p], make_float4(ex + slack, ey + slack, ez + slack, ph.w));
        node = p;
    }
}

// A node's child as the traversal sees it.  A child whose subtree holds at
// most leaf_size spheres (a single sphere included) is a leaf cluster:
// ref = its first sorted sphere, cnt = its sphere count; otherwise ref = its
// internal node index and cnt = 0.
struct PackedChild {
    float4 ctr, half;
    uint32_t ref, cnt;
};

__device__ PackedChild pack_child(int n, uint32_t leaf_size, const float4* node_ctr, const float4* node_half,
                                  const uint2* range, uint32_t c)
{
    PackedChild r;
    if (c >= (uint32_t)(n - 1)) {
        r.ref = c - (uint32_t)(n - 1);
        r.cnt = 1u;
    } else {
        const uint2 rg = range[c];
        const uint32_t size = rg.y - rg.x + 1u;
        r.ref = size <= leaf_size ? rg.x : c;
        r.cnt = size <= leaf_size ? size : 0u;
    }
    r.ctr = node_ctr[c];
    r.half = node_half[c];
    return r;
}

// 4-wide nodes for traversal: internal node i stores the boxes of its four
// grandchildren (a child that is a leaf cluster stands in for its own two
// slots, with an empty second slot: ref = ~0, cnt = 0), so one traversal step
// descends two levels of the binary tree.  Eight float4 rows (two 64-byte
// lines); rows 4j..4j+3 hold slots 2j and 2j+1 interleaved component by
// component, so one packed f32x2 instruction does a step of two box tests:
// (cx_a, cx_b, cy_a, cy_b), (cz_a, cz_b, hx_a, hx_b), (hy_a, hy_b, hz_a, hz_b),
// (ref_a, ref_b, cnt_a, cnt_b), with c the box centre and h its half extent.
// An internal slot's ref is a binary node index, whose own 4-wide node holds
// its grandchildren; nodes at odd depths are built but never visited.
__global__ void k_pack_quads(int n, uint32_t leaf_size, const float4* node_ctr, const float4* node_half,
                             const uint2* range, float4* quad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const uint32_t child[2] = {__float_as_uint(node_ctr[i].w), __float_as_uint(node_half[i].w)};
    for (int k = 0; k < 2; ++k) {
        const PackedChild c = pack_child(n, leaf_size, node_ctr, node_half, range, child[k]);
        PackedChild a = c, b;
        if (c.cnt == 0u) {
            a = pack_child(n, leaf_size, node_ctr, node_half, range, __float_as_uint(node_ctr[c.ref].w));
            b = pack_child(n, leaf_size, node_ctr, node_half, range, __float_as_uint(node_half[c.ref].w));
        } else {
            b.ctr = b.half = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            b.ref = 0xffffffffu;
            b.cnt = 0u;
        }
        float4* row = quad + 8 * (size_t)i + 4 * k;
        row[0] = make_float4(a.ctr.x, b.ctr.x, a.ctr.y, b.ctr.y);
        row[1] = make_float4(a.ctr.z, b.ctr.z, a.half.x, b.half.x);
        row[2] = make_float4(a.half.y, b.half.y, a.half.z, b.half.z);
        row[3] = make_float4(__uint_as_float(a.ref), __uint_as_float(b.ref), __uint_as_float(a.cnt),
                             __uint_as_float(b.cnt));
    }
}

}  // namespace

namespace {

// The scratch block's parts.  carve() both measures (base == nullptr) and
// assigns, so the size lbvh_bytes reports and the layout lbvh_build uses
// cannot disagree.
struct Parts {
    float4* node_ctr;
    float4* node_half;
    uint2* range;
    float4* quad;
    float4* leaf_sph;
    uint32_t* leaf_id;
    uint32_t *k0, *v0, *k1, *v1;
    uint32_t* parent;
    uint32_t* visits;
    uint32_t* counts;
    unsigned* bounds;
};

uint64_t carve(char* base, uint32_t n, Parts* q)
{
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) -> void* {
        void* r = base ? static_cast<void*>(base + off) : nullptr;
        off += (bytes + 255) & ~uint64_t(255);
        return r;
    };
    const uint64_t nn = n;
    const uint64_t blocks = (nn + kTile - 1) / kTile;
    q->node_ctr = static_cast<float4*>(take(2 * nn * sizeof(float4)));
    q->node_half = static_cast<float4*>(take(2 * nn * sizeof(float4)));
    q->range = static_cast<uint2*>(take(nn * sizeof(uint2)));
    q->quad = static_cast<float4*>(take(8 * nn * sizeof(float4)));
    q->leaf_sph = static_cast<float4*>(take(nn * sizeof(float4)));
    q->leaf_id = static_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    q->k0 = static_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    q->v0 = static_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    q->k1 = static_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    q->v1 = static_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    q->parent = static_cast<uint32_t*>(take(2 * nn * sizeof(uint32_t)));   // indexed by node, 2n-1 nodes
    q->visits = static_cast<uint32_t*>(take(nn * sizeof(uint32_t)));
    q->counts = static_cast<uint32_t*>(take(256 * blocks * sizeof(uint32_t)));
    q->bounds = static_cast<unsigned*>(take(6 * sizeof(unsigned)));
    return off;
}

__global__ void k_init_bounds(unsigned* bounds)
{
    if (threadIdx.x < 6) bounds[threadIdx.x] = threadIdx.x < 3 ? 0xffffffffu : 0u;
}

}  // namespace

uint64_t lbvh_bytes(uint32_t n)
{
    Parts q;
    return carve(nullptr, n ? n : 1, &q);
}

cudaError_t lbvh_build(const float4* sph, const float* radius, uint32_t n, uint32_t leaf_size, void* scratch,
                       uint64_t scratch_bytes, BvhView* out, cudaStream_t stream)
{
    if (n == 0 || scratch_bytes < lbvh_bytes(n)) return cudaErrorInvalidValue;
    Parts q;
    carve(static_cast<char*>(scratch), n, &q);
    const uint32_t blocks = (n + kTile - 1) / kTile;
    float4* node_ctr = q.node_ctr;
    float4* node_half = q.node_half;
    uint2* range = q.range;
    float4* leaf_sph = q.leaf_sph;
    uint32_t* leaf_id = q.leaf_id;
    uint32_t *k0 = q.k0, *v0 = q.v0, *k1 = q.k1, *v1 = q.v1;
    uint32_t* parent = q.parent;
    uint32_t* visits = q.visits;
    uint32_t* counts = q.counts;
    unsigned* bounds = q.bounds;

    k_init_bounds<<<1, 32, 0, stream>>>(bounds);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(visits, 0, (size_t)n * 4, stream);
    if (e != cudaSuccess) return e;
    const int g = (int)((n + kT - 1) / kT);
    k_bounds<<<g < 1024 ? g : 1024, kT, 0, stream>>>(sph, n, bounds);
    k_morton<<<g, kT, 0, stream>>>(sph, n, bounds, k0, v0);
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = pass * 8;
        k_sort_hist<<<blocks, kT, 0, stream>>>(k0, n, shift, counts);
        k_sort_scan<<<1, kT, 0, stream>>>(counts, 256u * blocks);
        k_sort_scatter<<<blocks, kT, 0, stream>>>(k0, v0, n, shift, counts, k1, v1);
        uint32_t* t = k0; k0 = k1; k1 = t;
        t = v0; v0 = v1; v1 = t;
    }
    k_gather_leaves<<<g, kT, 0, stream>>>(sph, radius, v0, (int)n, leaf_sph, leaf_id, node_ctr, node_half);
    if (n > 1) {
        const int gi = (int)((n - 1 + kT - 1) / kT);
        k_tree<<<gi, kT, 0, stream>>>(k0, (int)n, node_ctr, node_half, range, parent);
        k_refit<<<g, kT, 0, stream>>>((int)n, node_ctr, node_half, parent, visits);
        const uint32_t ls = leaf_size ? (leaf_size < 32u ? leaf_size : 32u) : 1u;   // clusters fit a 32-bit mask
        k_pack_quads<<<gi, kT, 0, stream>>>((int)n, ls, node_ctr, node_half, range, q.quad);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    out->node_ctr = node_ctr;
    out->node_half = node_half;
    out->node_range = range;
    out->quad = q.quad;
    out->leaf_sph = leaf_sph;
    out->leaf_id = leaf_id;
    out->n_leaves = n;
    out->leaf_size = leaf_size ? (leaf_size < 32u ? leaf_size : 32u) : 1u;
    out->root = 0;
    return cudaSuccess;
}

}  // namespace atx
