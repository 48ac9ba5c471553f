// rt_lbvh.cu — device-built LBVH, replacing the reference's per-frame octant binning
// (Model::RTPrepare, Model.cpp:402-480) and its brute-force octant lists (Model.cpp:748-811).
//
//   1. prep     per-triangle world box (p0+position, p0+e1, p0+e2) and centroid; the scene
//               box of all triangles by a block-reduced atomic min/max on order-preserving ints
//   2. morton   30-bit codes: 10 bits per axis of the centroid inside the scene box
//   3. sort     stable LSD radix sort of (code, index), 8-bit digits, 4 passes; each pass is a
//               per-tile digit histogram, one exclusive scan over (digit, tile), and a scatter
//               that ranks keys inside a tile with __match_any_sync so equal digits keep order
//   4. gather   triangles reordered to Morton order (p0|id, e1|obj, e2|mtl) and padded leaf boxes
//   5. karras   hierarchy from the sorted codes (Karras 2012), ties broken by index
//   6. refit    bottom-up boxes: the second child to arrive at a node (atomic counter) writes
//               the union of its children and moves up
// Nodes are 32 bytes: float4(min.xyz, left) and float4(max.xyz, right); internal nodes are
// 0..n-2, leaf k is node n-1+k.
#include <algorithm>

#include "rt_lbvh.cuh"

namespace rtg {

namespace {

constexpr int kTileKeys = 2048;   // keys per radix tile (256 threads x 8)
constexpr int kSortThreads = 256;

__device__ __forceinline__ unsigned f2ord(float f)
{
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

struct TriWorld {
    float p0[3], e1[3], e2[3], mn[3], mx[3];
};

__device__ __forceinline__ TriWorld leaf_world(const LbvhInput &in, int i)
{
    TriWorld w;
    if (i >= in.n) {   // sphere leaf: box = centre +- radius
        const int s = i - in.n;
        const float4 c = in.sph[s];
        const float r = in.sph_r[s];
        const float cc[3] = {c.x, c.y, c.z};
        for (int k = 0; k < 3; ++k) {
            w.p0[k] = cc[k], w.e1[k] = 0.0f, w.e2[k] = 0.0f;
            w.mn[k] = __fsub_rn(cc[k], r);
            w.mx[k] = __fadd_rn(cc[k], r);
        }
        return w;
    }
    const float *p = in.tri_p + 9ll * i;
    const float *pos = in.obj_pos + 3ll * in.tri_obj[i];
    for (int k = 0; k < 3; ++k) {
        w.p0[k] = __fadd_rn(p[k], pos[k]);           // clTri::p0 = p0 + position
        w.e1[k] = __fsub_rn(p[3 + k], p[k]);          // axisu = p1 - p0 (model space)
        w.e2[k] = __fsub_rn(p[6 + k], p[k]);          // axisv = p2 - p0
        float a = w.p0[k], b = __fadd_rn(w.p0[k], w.e1[k]), c = __fadd_rn(w.p0[k], w.e2[k]);
        w.mn[k] = fminf(a, fminf(b, c));
        w.mx[k] = fmaxf(a, fmaxf(b, c));
    }
    return w;
}

__global__ void k_prep(LbvhInput in, float4 *centroid, unsigned *box)
{
    __shared__ unsigned smn[3], smx[3];
    if (threadIdx.x < 3) smn[threadIdx.x] = 0xffffffffu, smx[threadIdx.x] = 0u;
    __syncthreads();
    unsigned lmn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, lmx[3] = {0u, 0u, 0u};
    const int total = in.n + in.n_sph;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        TriWorld w = leaf_world(in, i);
        float c[3];
        for (int k = 0; k < 3; ++k) {
            c[k] = __fmul_rn(__fadd_rn(w.mn[k], w.mx[k]), 0.5f);
            lmn[k] = min(lmn[k], f2ord(w.mn[k]));
            lmx[k] = max(lmx[k], f2ord(w.mx[k]));
        }
        centroid[i] = make_float4(c[0], c[1], c[2], 0.0f);
    }
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            lmn[k] = min(lmn[k], __shfl_xor_sync(0xffffffffu, lmn[k], off));
            lmx[k] = max(lmx[k], __shfl_xor_sync(0xffffffffu, lmx[k], off));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&smn[k], lmn[k]);
            atomicMax(&smx[k], lmx[k]);
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        atomicMin(&box[threadIdx.x], smn[threadIdx.x]);
        atomicMax(&box[3 + threadIdx.x], smx[threadIdx.x]);
    }
}

__device__ __forceinline__ unsigned expand10(unsigned v)
{
    v &= 0x3ffu;
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// 30-bit codes: 10 bits per axis of the leaf centre, quantised over the scene box with one
// scale for all three axes, the box's largest extent / 1024 (cubic cells). Per-axis scales
// would spend the top bits of a flat scene's short axis first: a 40 x 4 x 40 terrain's second
// split would cut it by height into two halves that both span the whole footprint. Cubic
// cells split the long axes first; on config 2 that is 24-29 % fewer node visits.
__global__ void k_morton(int n, const float4 *centroid, const unsigned *box, unsigned *codes, unsigned *idx)
{
    float mn[3], ext[3];
    for (int k = 0; k < 3; ++k) {
        mn[k] = ord2f(box[k]);
        ext[k] = __fsub_rn(ord2f(box[3 + k]), mn[k]);
    }
    const float emax = fmaxf(ext[0], fmaxf(ext[1], ext[2]));
    const float s = emax > 0.0f ? __fdiv_rn(1024.0f, emax) : 0.0f;
    const float scale[3] = {s, s, s};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 c = centroid[i];
        float cc[3] = {c.x, c.y, c.z};
        unsigned q[3];
        for (int k = 0; k < 3; ++k) {
            float f = __fmul_rn(__fsub_rn(cc[k], mn[k]), scale[k]);
            int qi = (int)f;
            q[k] = (unsigned)min(max(qi, 0), 1023);
        }
        codes[i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
        idx[i] = (unsigned)i;
    }
}

// ---- radix sort --------------------------------------------------------------------------------
__global__ void __launch_bounds__(kSortThreads) k_hist(int n, const unsigned *keys, int shift, unsigned *hist, int tiles)
{
    __shared__ unsigned h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int tile = blockIdx.x;
    const int start = tile * kTileKeys;
    for (int r = 0; r < kTileKeys / kSortThreads; ++r) {
        int i = start + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + tile] = h[threadIdx.x];
}

// Exclusive scan of the digit-major tile histograms (m = 256 x tiles counts) in three steps:
// block sums of 4096-count chunks, one block scanning those sums, then each chunk scanned in its
// block with the chunk's offset added. Loads are coalesced (a block reads its chunk as 1024 x
// uint4), so a pass costs a few microseconds instead of one block walking the whole array.
constexpr int kScanThreads = 1024, kScanChunk = 4 * kScanThreads;
__host__ __device__ constexpr int scan_chunks(int m) { return (m + kScanChunk - 1) / kScanChunk; }

// the block's inclusive prefix of v (blockDim.x == kScanThreads); *total = the block's sum
__device__ __forceinline__ unsigned block_inclusive_scan(unsigned v, unsigned *warp_sums, unsigned *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += u;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned w = warp_sums[lane];
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned u = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += u;
        }
        warp_sums[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    if (total) *total = warp_sums[31];
    return v + (warp > 0 ? warp_sums[warp - 1] : 0u);
}

// m is a multiple of 4 (256 counts per tile), so a thread's 4 counts are one aligned uint4
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const unsigned *a, int m, unsigned *part)
{
    __shared__ unsigned warp_sums[32];
    const int i = blockIdx.x * kScanChunk + 4 * threadIdx.x;
    unsigned v = 0;
    if (i < m) {
        const uint4 q = *reinterpret_cast<const uint4 *>(a + i);
        v = q.x + q.y + q.z + q.w;
    }
    unsigned total = 0;
    block_inclusive_scan(v, warp_sums, &total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// exclusive scan of the chunk sums in place (one block, any number of chunks)
__global__ void __launch_bounds__(kScanThreads) k_scan_top(unsigned *part, int chunks)
{
    __shared__ unsigned warp_sums[32];
    unsigned carry = 0;
    for (int base = 0; base < chunks; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const unsigned v = i < chunks ? part[i] : 0u;
        unsigned total = 0;
        const unsigned inc = block_inclusive_scan(v, warp_sums, &total);
        if (i < chunks) part[i] = carry + inc - v;
        carry += total;
        __syncthreads();   // warp_sums is reused by the next round
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(unsigned *a, int m, const unsigned *part)
{
    __shared__ unsigned warp_sums[32];
    const int i = blockIdx.x * kScanChunk + 4 * threadIdx.x;
    uint4 q = make_uint4(0, 0, 0, 0);
    if (i < m) q = *reinterpret_cast<const uint4 *>(a + i);
    const unsigned t = q.x + q.y + q.z + q.w;
    const unsigned excl = block_inclusive_scan(t, warp_sums, nullptr) - t + part[blockIdx.x];
    if (i < m) {
        uint4 o;
        o.x = excl;
        o.y = o.x + q.x;
        o.z = o.y + q.y;
        o.w = o.z + q.z;
        *reinterpret_cast<uint4 *>(a + i) = o;
    }
}

__global__ void __launch_bounds__(kSortThreads) k_scatter(int n, const unsigned *kin, const unsigned *vin, unsigned *kout,
                                                          unsigned *vout, int shift, const unsigned *hist, int tiles)
{
    __shared__ unsigned wcount[kSortThreads / 32][257];
    __shared__ unsigned base[256];
    __shared__ unsigned round_total[256];
    const int tile = blockIdx.x, start = tile * kTileKeys;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    base[threadIdx.x] = hist[threadIdx.x * tiles + tile];
    for (int w = 0; w < kSortThreads / 32; ++w) wcount[w][threadIdx.x] = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kSortThreads / 32; ++w) wcount[w][256] = 0;
    __syncthreads();
    for (int r = 0; r < kTileKeys / kSortThreads; ++r) {
        const int i = start + r * kSortThreads + threadIdx.x;
        const bool ok = i < n;
        unsigned key = 0, val = 0, d = 256;
        if (ok) {
            key = kin[i];
            val = vin[i];
            d = (key >> shift) & 0xffu;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned wrank = __popc(peers & lt);
        if (wrank == 0) wcount[warp][d] = __popc(peers);
        __syncthreads();
        {   // exclusive prefix over warps for each digit
            unsigned run = 0;
            for (int w = 0; w < kSortThreads / 32; ++w) {
                unsigned c = wcount[w][threadIdx.x];
                wcount[w][threadIdx.x] = run;
                run += c;
            }
            round_total[threadIdx.x] = run;
        }
        __syncthreads();
        if (ok) {
            const unsigned dst = base[d] + wcount[warp][d] + wrank;
            kout[dst] = key;
            vout[dst] = val;
        }
        __syncthreads();
        base[threadIdx.x] += round_total[threadIdx.x];
        for (int w = 0; w < kSortThreads / 32; ++w) wcount[w][threadIdx.x] = 0;
        __syncthreads();
    }
}

// ---- gather, hierarchy, refit -------------------------------------------------------------------
__global__ void k_gather(LbvhInput in, LbvhOutput out, const unsigned *perm, const unsigned *box)
{
    const int n = in.n + in.n_sph;
    // absolute padding from the scene size: 2^-20 of its largest coordinate magnitude
    float scene_mag = 0.0f;
    for (int k = 0; k < 6; ++k) scene_mag = fmaxf(scene_mag, fabsf(ord2f(box[k])));
    const float pad_abs = scene_mag * (1.0f / 1048576.0f);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = (int)perm[k];
        TriWorld w = leaf_world(in, i);
        if (i < in.n) {
            out.tri[3ll * k] = make_float4(w.p0[0], w.p0[1], w.p0[2], __int_as_float(in.tri_id[i]));
            out.tri[3ll * k + 1] = make_float4(w.e1[0], w.e1[1], w.e1[2], __int_as_float(in.tri_obj[i]));
            int m = in.tri_mtl[i];
            if (in.bad && (m < 0 || m >= in.n_mtl)) {   // rejected by the caller; never read out of range
                atomicOr(in.bad, 1);
                m = 0;
            }
            out.tri[3ll * k + 2] = make_float4(w.e2[0], w.e2[1], w.e2[2], __int_as_float(m));
            const float *nn = in.tri_n + 9ll * i;
            for (int j = 0; j < 3; ++j) out.trin[3ll * k + j] = make_float4(nn[3 * j], nn[3 * j + 1], nn[3 * j + 2], 0.0f);
            if (out.triuv) {
                const float *uv = in.tri_uv ? in.tri_uv + 6ll * i : nullptr;
                for (int j = 0; j < 3; ++j) out.triuv[3ll * k + j] = uv ? make_float2(uv[2 * j], uv[2 * j + 1]) : make_float2(0, 0);
            }
        } else {
            const int sidx = i - in.n;
            out.tri[3ll * k] = in.sph[sidx];
            out.tri[3ll * k + 1] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(in.sph_obj[sidx]));
            out.tri[3ll * k + 2] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1 - in.sph_prim[sidx]));
            for (int j = 0; j < 3; ++j) out.trin[3ll * k + j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (out.triuv)
                for (int j = 0; j < 3; ++j) out.triuv[3ll * k + j] = make_float2(0, 0);
        }
        // padded leaf box: the exact triangle test may accept a hit a few ulps outside
        float mag = 0.0f, ext = 0.0f;
        for (int j = 0; j < 3; ++j) {
            mag = fmaxf(mag, fmaxf(fabsf(w.mn[j]), fabsf(w.mx[j])));
            ext = fmaxf(ext, w.mx[j] - w.mn[j]);
        }
        const float pad = (mag + ext) * (1.0f / 65536.0f) + pad_abs;
        const long long node = (long long)(n - 1) + k;
        out.nodes[2 * node] = make_float4(w.mn[0] - pad, w.mn[1] - pad, w.mn[2] - pad, __int_as_float(-1));
        out.nodes[2 * node + 1] = make_float4(w.mx[0] + pad, w.mx[1] + pad, w.mx[2] + pad, __int_as_float(-1));
    }
}

__device__ __forceinline__ int delta(const unsigned *codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const unsigned a = codes[i], b = codes[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((unsigned)i ^ (unsigned)j);
}

__global__ void k_karras(int n, const unsigned *codes, float4 *nodes, int *parent)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
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
        for (int div = 2;; div <<= 1) {
            const int t = (l + div - 1) / div;
            if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
            if (t <= 1) break;
        }
        const int gamma = i + s * d + min(d, 0);
        const int left = (min(i, j) == gamma) ? (n - 1) + gamma : gamma;
        const int right = (max(i, j) == gamma + 1) ? (n - 1) + gamma + 1 : gamma + 1;
        nodes[2ll * i].w = __int_as_float(left);
        nodes[2ll * i + 1].w = __int_as_float(right);
        parent[left] = i;
        parent[right] = i;
        if (i == 0) parent[0] = -1;
    }
}

__global__ void k_refit(int n, float4 *nodes, const int *parent, int *flags)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int node = (n - 1) + k;
        int p = parent[node];
        for (int depth = 0; p >= 0 && p < n - 1 && depth < 128; ++depth) {
            __threadfence();
            if (atomicAdd(&flags[p], 1) == 0) break;   // first child: the sibling finishes the node
            const float4 lo = nodes[2ll * p], hi = nodes[2ll * p + 1];
            const int c0 = __float_as_int(lo.w), c1 = __float_as_int(hi.w);
            const float4 a0 = __ldcg(&nodes[2ll * c0]), a1 = __ldcg(&nodes[2ll * c0 + 1]);
            const float4 b0 = __ldcg(&nodes[2ll * c1]), b1 = __ldcg(&nodes[2ll * c1 + 1]);
            __stcg(&nodes[2ll * p], make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), lo.w));
            __stcg(&nodes[2ll * p + 1], make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), hi.w));
            node = p;
            p = parent[p];
        }
    }
}

// A 4-wide node for every internal node i: the slots are i's grandchildren — each child's two
// children when the child is internal, the child itself when it is a leaf — and when a leaf
// child leaves a slot free, the internal grandchild with the largest surface area is replaced
// by its two children. Every internal slot is thus two or three binary levels below i: a path
// of at most 63 binary levels takes at most 32 four-wide steps of at most 3 pushes each.
// Traversal starts at the root and steps from a node to its slots (every internal node has a
// record, so any descendant can be a slot).
// Record (128 B, one line): float4 lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4], then
// int4 refs (>= 0 internal node, < 0 leaf ~k, kEmptySlot unused), then padding. An unused
// slot's box is the point (1e38, 1e38, 1e38), which no ray reaches within a cull distance.
__device__ __forceinline__ float half_area(const float4 *nodes, int x)
{
    const float4 l = __ldcg(&nodes[2ll * x]), h = __ldcg(&nodes[2ll * x + 1]);
    const float dx = h.x - l.x, dy = h.y - l.y, dz = h.z - l.z;
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_quads(int n, const float4 *nodes, float4 *quads)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        int slot[4];
        int k = 0;
        const int c[2] = {__float_as_int(nodes[2ll * i].w), __float_as_int(nodes[2ll * i + 1].w)};
        for (int j = 0; j < 2; ++j) {
            if (c[j] >= n - 1) {
                slot[k++] = c[j];
            } else {
                slot[k++] = __float_as_int(__ldcg(&nodes[2ll * c[j]]).w);
                slot[k++] = __float_as_int(__ldcg(&nodes[2ll * c[j] + 1]).w);
            }
        }
        if (k == 3) {   // one leaf child: split the largest internal grandchild
            int best = -1;
            float area = -1.0f;
            for (int j = 0; j < 3; ++j)
                if (slot[j] < n - 1) {
                    const float a = half_area(nodes, slot[j]);
                    if (a > area) area = a, best = j;
                }
            if (best >= 0) {
                const int x = slot[best];
                slot[best] = __float_as_int(__ldcg(&nodes[2ll * x]).w);
                slot[k++] = __float_as_int(__ldcg(&nodes[2ll * x + 1]).w);
            }
        }
        float lo[3][4], hi[3][4];
        int ref[4];
        for (int j = 0; j < 4; ++j) {
            if (j < k) {
                const int x = slot[j];
                const float4 l = __ldcg(&nodes[2ll * x]), h = __ldcg(&nodes[2ll * x + 1]);
                lo[0][j] = l.x, lo[1][j] = l.y, lo[2][j] = l.z;
                hi[0][j] = h.x, hi[1][j] = h.y, hi[2][j] = h.z;
                ref[j] = x >= n - 1 ? ~(x - (n - 1)) : x;
            } else {   // a point at 1e38: its entry distance exceeds every cull (<= 1e20)
                for (int a = 0; a < 3; ++a) lo[a][j] = hi[a][j] = 1e38f;
                ref[j] = kEmptySlot;
            }
        }
        float4 *q = quads + 8ll * i;
        for (int a = 0; a < 3; ++a) {
            q[2 * a] = make_float4(lo[a][0], lo[a][1], lo[a][2], lo[a][3]);
            q[2 * a + 1] = make_float4(hi[a][0], hi[a][1], hi[a][2], hi[a][3]);
        }
        q[6] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), __int_as_float(ref[2]), __int_as_float(ref[3]));
        q[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// ---- clustering build (PLOC: Meister & Bittner, "Parallel Locally-Ordered Clustering for
// Bounding Volume Hierarchy Construction", 2018) ----------------------------------------------
// Clusters start as the leaves in Morton order. Each round every cluster finds its nearest
// neighbour among the kPlocRadius clusters on either side (distance: half the surface area of
// the union of the two boxes; equal distances go to the lower index, which orders all pairs by
// (distance, lower index, higher index), so the closest pair of a round is always mutual), each
// mutual pair merges into a new internal node in the lower cluster's place, and the survivors
// are compacted in order. Internal nodes are numbered L-2, L-3, ... in merge order, so the last
// merge — the root — is node 0, as in the Karras layout; no refit is needed.
constexpr int kPlocRadius = 16;
constexpr int kPlocThreads = 256;

// in units of the scene's largest extent (inv = its reciprocal), so that no product overflows
__device__ __forceinline__ float union_half_area(float4 alo, float4 ahi, float4 blo, float4 bhi, float inv)
{
    const float dx = (fmaxf(ahi.x, bhi.x) - fminf(alo.x, blo.x)) * inv;
    const float dy = (fmaxf(ahi.y, bhi.y) - fminf(alo.y, blo.y)) * inv;
    const float dz = (fmaxf(ahi.z, bhi.z) - fminf(alo.z, blo.z)) * inv;
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_ploc_init(int L, const float4 *nodes, int *id, float4 *lo, float4 *hi, int *counts)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) counts[1] = L;   // cluster count before the first merge pass
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
        const long long x = (long long)(L - 1) + k;
        id[k] = (int)x;
        lo[k] = __ldcg(&nodes[2 * x]);
        hi[k] = __ldcg(&nodes[2 * x + 1]);
    }
}

// m_in: this round's cluster count (device); the grid covers an upper bound of it
__global__ void __launch_bounds__(kPlocThreads) k_ploc_nn(const int *m_in, const unsigned *box, const float4 *lo,
                                                          const float4 *hi, int *nn)
{
    const int m = *m_in;
    float emax = 0.0f;
    for (int k = 0; k < 3; ++k) emax = fmaxf(emax, ord2f(box[3 + k]) - ord2f(box[k]));
    const float inv = emax > 0.0f && emax < INFINITY ? 1.0f / emax : 1.0f;
    constexpr int W = kPlocThreads + 2 * kPlocRadius;
    __shared__ float4 slo[W], shi[W];
    const int base = blockIdx.x * kPlocThreads - kPlocRadius;
    for (int k = threadIdx.x; k < W; k += kPlocThreads) {
        const int g = base + k;
        if (g >= 0 && g < m) slo[k] = lo[g], shi[k] = hi[g];
    }
    __syncthreads();
    const int i = blockIdx.x * kPlocThreads + threadIdx.x;
    if (i >= m) return;
    const int si = threadIdx.x + kPlocRadius;
    float best = INFINITY;
    int bj = -1;
    for (int r = -kPlocRadius; r <= kPlocRadius; ++r) {   // increasing j: the first of equals wins
        const int j = i + r;
        if (r == 0 || j < 0 || j >= m) continue;
        const float d = union_half_area(slo[si], shi[si], slo[si + r], shi[si + r], inv);
        if (d < best) best = d, bj = j;
    }
    nn[i] = bj;
}

// merge mutual pairs into `out` (uncompacted, the pair in its lower slot); pos[i] = survives
__global__ void k_ploc_merge(const int *m_in, int m4, int L, const int *nn, const int *id, const float4 *lo, const float4 *hi,
                             int *oid, float4 *olo, float4 *ohi, unsigned *valid, unsigned *pos, int *counts, float4 *nodes,
                             int *parent)
{
    // whole warps iterate together (the bound is rounded up to a warp), so a warp's merges take
    // their node numbers with one atomic (a counter every merge hit at once serialised). m4 is
    // a bound of this round's count rounded up to 4: the scan reads zeros beyond the count.
    const int m = *m_in;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long top = ((long long)m4 + 31) & ~31ll;
    const int lane = threadIdx.x & 31;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g - lane < top; g += stride) {
        const int i = (int)g;
        const int j = i < m ? nn[i] : -1;
        const bool mutual = i < m && j >= 0 && nn[j] == i;
        const bool merge = mutual && i < j;
        const unsigned b = __ballot_sync(0xffffffffu, merge);
        int base = 0;
        if (lane == 0 && b) base = atomicAdd(&counts[0], __popc(b));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (i >= m4) continue;
        if (i >= m) {
            pos[i] = 0;
            continue;
        }
        if (mutual && i > j) {   // merged into j
            valid[i] = pos[i] = 0;
            continue;
        }
        if (merge) {
            const int x = L - 2 - (base + __popc(b & ((1u << lane) - 1u)));
            const float4 a = lo[i], bl = lo[j], c = hi[i], d = hi[j];
            const float4 l = make_float4(fminf(a.x, bl.x), fminf(a.y, bl.y), fminf(a.z, bl.z), __int_as_float(id[i]));
            const float4 h = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), __int_as_float(id[j]));
            nodes[2ll * x] = l;
            nodes[2ll * x + 1] = h;
            parent[id[i]] = x;
            parent[id[j]] = x;
            oid[i] = x;
            olo[i] = l;
            ohi[i] = h;
        } else {
            oid[i] = id[i];
            olo[i] = lo[i];
            ohi[i] = hi[i];
        }
        valid[i] = pos[i] = 1;
    }
}

__global__ void k_ploc_compact(const int *m_in, const unsigned *valid, const unsigned *pos, const int *id,
                               const float4 *lo, const float4 *hi, int *oid, float4 *olo, float4 *ohi, int *m_out)
{
    const int m = *m_in;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        if (valid[i]) {
            const unsigned p = pos[i];
            oid[p] = id[i];
            olo[p] = lo[i];
            ohi[p] = hi[i];
        }
        if (i == m - 1) *m_out = (int)(pos[i] + valid[i]);
    }
}

// the deepest leaf of a clustered tree (root = node 0), into counts[3]; a walk longer than 4096
// steps (no tree built here is) counts as 4096
__global__ void k_ploc_depth(int L, const int *parent, int *counts)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
        int x = L - 1 + k, d = 0;
        while (x != 0 && d < 4096) {
            x = parent[x];
            ++d;
        }
        atomicMax(&counts[3], d);
    }
}

struct Scratch {
    unsigned *box;        // 8
    float4 *centroid;     // n
    unsigned *codes[2];   // n each
    unsigned *idx[2];     // n each
    unsigned *hist;       // 256 * tiles
    unsigned *part;       // scan_chunks(256 * tiles) chunk sums of the histogram scan
    int *parent;          // 2n - 1
    int *flags;           // n - 1
    // clustering build: clusters (node id, box) double-buffered, nearest neighbours, survivor
    // flags and their scan, the scan's chunk sums, the merge counter and the survivor count
    int *cl_id[2];
    float4 *cl_lo[2], *cl_hi[2];
    int *nn;
    unsigned *valid, *pos, *pos_part;
    int *counts;          // [0] merges so far, [1] survivors of the last round
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

Scratch carve(void *base, int n)
{
    const int tiles = (n + kTileKeys - 1) / kTileKeys;
    char *p = (char *)base;
    Scratch s;
    s.box = (unsigned *)p;
    p += 256;
    s.centroid = (float4 *)p;
    p += align256(sizeof(float4) * (size_t)n);
    for (int k = 0; k < 2; ++k) {
        s.codes[k] = (unsigned *)p;
        p += align256(4 * (size_t)n);
        s.idx[k] = (unsigned *)p;
        p += align256(4 * (size_t)n);
    }
    s.hist = (unsigned *)p;
    p += align256(4 * 256 * (size_t)tiles);
    s.part = (unsigned *)p;
    p += align256(4 * (size_t)scan_chunks(256 * tiles));
    s.parent = (int *)p;
    p += align256(4 * (size_t)(2 * n));
    s.flags = (int *)p;
    p += align256(4 * (size_t)n);
    for (int k = 0; k < 2; ++k) {
        s.cl_id[k] = (int *)p;
        p += align256(4 * (size_t)n);
        s.cl_lo[k] = (float4 *)p;
        p += align256(16 * (size_t)n);
        s.cl_hi[k] = (float4 *)p;
        p += align256(16 * (size_t)n);
    }
    s.nn = (int *)p;
    p += align256(4 * (size_t)n);
    s.valid = (unsigned *)p;
    p += align256(4 * (size_t)n);
    s.pos = (unsigned *)p;
    p += align256(4 * ((size_t)n + 4));
    s.pos_part = (unsigned *)p;
    p += align256(4 * (size_t)scan_chunks(n + 4));
    s.counts = (int *)p;
    return s;
}

int grid_of(long long n, int block)
{
    long long g = (n + block - 1) / block;
    return (int)std::max<long long>(1, std::min<long long>(g, 65535));
}

// sorted codes end in codes[0] / idx[0] after an even number of passes
cudaError_t morton_and_sort(const LbvhInput &in, const Scratch &sc, cudaStream_t s)
{
    const int n = in.n + in.n_sph;
    const int tiles = (n + kTileKeys - 1) / kTileKeys;
    cudaError_t e = cudaMemsetAsync(sc.box, 0xff, 12, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sc.box + 3, 0, 12, s);
    if (e != cudaSuccess) {
        g_build_step = "scene box";
        return e;
    }
    k_prep<<<grid_of(n, 256), 256, 0, s>>>(in, sc.centroid, sc.box);
    k_morton<<<grid_of(n, 256), 256, 0, s>>>(n, sc.centroid, sc.box, sc.codes[0], sc.idx[0]);
    {
        const cudaError_t r = cudaGetLastError();
        if (r != cudaSuccess) {
            g_build_step = "Morton codes";
            return r;
        }
    }
    for (int pass = 0; pass < 4; ++pass) {
        const int src = pass & 1, dst = src ^ 1;
        k_hist<<<tiles, kSortThreads, 0, s>>>(n, sc.codes[src], 8 * pass, sc.hist, tiles);
        const int m = 256 * tiles, chunks = scan_chunks(m);
        k_scan_reduce<<<chunks, kScanThreads, 0, s>>>(sc.hist, m, sc.part);
        k_scan_top<<<1, kScanThreads, 0, s>>>(sc.part, chunks);
        k_scan_down<<<chunks, kScanThreads, 0, s>>>(sc.hist, m, sc.part);
        k_scatter<<<tiles, kSortThreads, 0, s>>>(n, sc.codes[src], sc.idx[src], sc.codes[dst], sc.idx[dst], 8 * pass,
                                                 sc.hist, tiles);
        const cudaError_t r = cudaGetLastError();
        if (r != cudaSuccess) {
            g_build_step = "radix sort";
            return r;
        }
    }
    return cudaSuccess;
}

} // namespace

__global__ void k_tri_objects(const int *ranges, int n_ranges, int n, int *obj, int *ids)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = n_ranges - 1;
        while (lo < hi) {   // last range whose first <= i
            const int mid = (lo + hi + 1) >> 1;
            if (ranges[3 * mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        obj[i] = ranges[3 * lo + 2];
        if (ids) ids[i] = i - ranges[3 * lo];
    }
}

void launch_tri_objects(const int *ranges, int n_ranges, int n, int *obj, int *ids, cudaStream_t s)
{
    if (n <= 0 || n_ranges <= 0) return;
    k_tri_objects<<<grid_of(n, 256), 256, 0, s>>>(ranges, n_ranges, n, obj, ids);
}

size_t lbvh_scratch_bytes(int n)
{
    const int tiles = (n + kTileKeys - 1) / kTileKeys;
    return 256 + align256(sizeof(float4) * (size_t)n) + 4 * align256(4 * (size_t)n) + align256(4 * 256 * (size_t)tiles) +
           align256(4 * (size_t)scan_chunks(256 * tiles)) + align256(4 * (size_t)(2 * n)) + align256(4 * (size_t)n) +
           2 * (align256(4 * (size_t)n) + 2 * align256(16 * (size_t)n)) + 2 * align256(4 * (size_t)n) +
           align256(4 * ((size_t)n + 4)) + align256(4 * (size_t)scan_chunks(n + 4)) + 256 + 256;
}

cudaError_t lbvh_morton_sort(const LbvhInput &in, uint32_t *codes_out, uint32_t *perm_out, void *scratch, cudaStream_t s)
{
    const int n = in.n + in.n_sph;
    if (n <= 0) return cudaSuccess;
    Scratch sc = carve(scratch, n);
    cudaError_t e = morton_and_sort(in, sc, s);
    if (e != cudaSuccess) return e;
    cudaMemcpyAsync(codes_out, sc.codes[0], 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(perm_out, sc.idx[0], 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
    return cudaGetLastError();
}

const char *g_build_step = "";   // the build step that failed last (diagnostics)

cudaError_t lbvh_build(const LbvhInput &in, const LbvhOutput &out, void *scratch, cudaStream_t s,
                       cudaEvent_t shading_ready)
{
    const int n = in.n + in.n_sph;
    if (n <= 0) return cudaSuccess;
    Scratch sc = carve(scratch, n);
    cudaError_t e = morton_and_sort(in, sc, s);
    if (e != cudaSuccess) return e;
    auto step = [&](const char *name) {
        cudaError_t r = cudaGetLastError();
        if (r != cudaSuccess) g_build_step = name;
        return r;
    };
    if (shading_ready && (e = cudaStreamWaitEvent(s, shading_ready, 0)) != cudaSuccess) return e;
    k_gather<<<grid_of(n, 256), 256, 0, s>>>(in, out, sc.idx[0], sc.box);
    if ((e = step("gather")) != cudaSuccess) return e;
    if (n > 1 && in.cluster_count) {
        // clustering build. The cluster count stays on the device (round r reads slot 1 + r % 2
        // and writes the other); kernels are sized by the last count the host read, which bounds
        // it. The host reads the count after every round while clusters are many (those rounds
        // are long) and after every 8 rounds when they are few (a round trip each would cost
        // more than the rounds).
        cudaMemsetAsync(sc.counts, 0, 16, s);
        k_ploc_init<<<grid_of(n, 256), 256, 0, s>>>(n, out.nodes, sc.cl_id[0], sc.cl_lo[0], sc.cl_hi[0], sc.counts);
        int mh = n, r = 0;
        bool stuck = false;   // rounds without a merge (distances that do not order, e.g. NaN)
        while (true) {
            const int rounds = mh > 65536 ? 1 : 8;
            for (int q = 0; q < rounds; ++q, ++r) {
                const int *m_in = sc.counts + 1 + (r & 1);
                int *m_out = sc.counts + 1 + ((r + 1) & 1);
                const int m4 = (mh + 3) & ~3;
                k_ploc_nn<<<(mh + kPlocThreads - 1) / kPlocThreads, kPlocThreads, 0, s>>>(m_in, sc.box, sc.cl_lo[0],
                                                                                        sc.cl_hi[0], sc.nn);
                k_ploc_merge<<<grid_of(m4, 256), 256, 0, s>>>(m_in, m4, n, sc.nn, sc.cl_id[0], sc.cl_lo[0], sc.cl_hi[0],
                                                              sc.cl_id[1], sc.cl_lo[1], sc.cl_hi[1], sc.valid, sc.pos,
                                                              sc.counts, out.nodes, sc.parent);
                const int chunks = scan_chunks(m4);
                k_scan_reduce<<<chunks, kScanThreads, 0, s>>>(sc.pos, m4, sc.pos_part);
                k_scan_top<<<1, kScanThreads, 0, s>>>(sc.pos_part, chunks);
                k_scan_down<<<chunks, kScanThreads, 0, s>>>(sc.pos, m4, sc.pos_part);
                k_ploc_compact<<<grid_of(mh, 256), 256, 0, s>>>(m_in, sc.valid, sc.pos, sc.cl_id[1], sc.cl_lo[1],
                                                               sc.cl_hi[1], sc.cl_id[0], sc.cl_lo[0], sc.cl_hi[0], m_out);
            }
            if ((e = step("clustering")) != cudaSuccess) return e;
            if ((e = cudaMemcpyAsync(in.cluster_count, sc.counts + 1 + (r & 1), sizeof(int), cudaMemcpyDeviceToHost, s)) !=
                    cudaSuccess ||
                (e = cudaStreamSynchronize(s)) != cudaSuccess)
                return e;
            const int m = *in.cluster_count;
            if (m <= 1) break;
            if (m >= mh) {   // every round with two or more clusters merges its closest pair
                stuck = true;
                break;
            }
            mh = m;
        }
        // traversal keeps 96 stack entries, enough for trees of depth 63: a deeper clustered tree
        // (or one the rounds could not finish) is replaced by the radix tree, which never is
        if (!stuck) k_ploc_depth<<<grid_of(n, 256), 256, 0, s>>>(n, sc.parent, sc.counts);
        if ((e = step("clustering depth")) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(in.cluster_count, sc.counts + 3, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return e;
        if (!stuck && *in.cluster_count <= 63) {
            if (out.quads) k_quads<<<grid_of(n - 1, 256), 256, 0, s>>>(n, out.nodes, out.quads);
            return step("4-wide nodes");
        }
    }
    if (n > 1) {
        k_karras<<<grid_of(n - 1, 256), 256, 0, s>>>(n, sc.codes[0], out.nodes, sc.parent);
        if ((e = step("hierarchy")) != cudaSuccess) return e;
        cudaMemsetAsync(sc.flags, 0, 4 * (size_t)(n - 1), s);
        k_refit<<<grid_of(n, 256), 256, 0, s>>>(n, out.nodes, sc.parent, sc.flags);
        if ((e = step("refit")) != cudaSuccess) return e;
        if (out.quads) k_quads<<<grid_of(n - 1, 256), 256, 0, s>>>(n, out.nodes, out.quads);
        if ((e = step("4-wide nodes")) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

} // namespace rtg

// ---- allocation-free Morton sort -------------------------------------------------------------
// Working memory of rt_morton_sort_noalloc: one fixed array in device memory, sized for
// RT_NOALLOC_MAX_TRIS triangles (centroids 16 B, second sort buffer 8 B and zero object ids
// 4 B per triangle, digit histograms 1 KB per 2048 triangles and 4 B per 4096 histogram counts
// for their scan, the scene box and a zero object position). Every GPU that loads the library
// holds it until the process exits.
#include <cstdio>

#include "../../include/rt_gb300.h"

namespace rtg {
namespace {

constexpr size_t kNoAllocN = (size_t)RT_NOALLOC_MAX_TRIS;
constexpr size_t kNoAllocTiles = (kNoAllocN + kTileKeys - 1) / kTileKeys;
constexpr size_t kNoAllocChunks = (256 * kNoAllocTiles + 4095) / 4096;   // histogram-scan chunk sums
constexpr size_t kNoAllocBytes = 256 + 256 + 16 * kNoAllocN + 4 * kNoAllocN + 4 * kNoAllocN + 4 * kNoAllocN +
                                 1024 * kNoAllocTiles + 4 * kNoAllocChunks;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

} // namespace
} // namespace rtg

// Callers that cannot allocate device memory: a plugin inside a host application whose
// device memory is owned and budgeted by that application, or code on a latency-bound path
// where cudaMalloc / cudaFree would block on the device. They pass device buffers they
// already own; this entry point uses only the fixed array above (no cudaMalloc, cudaFree or
// allocating library call). Every call looks up the array's device address on the current
// device (cudaGetSymbolAddress): an address kept from an earlier call would dangle after a
// cudaDeviceReset, which reloads the module. The first call on a device loads the module
// there; make that first call before any stream capture. All calls share the one array,
// which keeps the last call's contents: calls that overlap on the GPU (two streams, two
// threads) race and corrupt each other's results, so serialise them.
extern "C" int rt_morton_sort_noalloc(const float *d_tri_p, int64_t n_tris, uint32_t *d_codes, uint32_t *d_perm,
                                      void *cuda_stream)
{
    using namespace rtg;
    if (n_tris < 0 || (n_tris > 0 && (!d_tri_p || !d_codes || !d_perm))) return RT_ERR_INVALID;
    if (n_tris > (int64_t)RT_NOALLOC_MAX_TRIS) {
        std::fprintf(stderr, "rt_morton_sort_noalloc: %lld triangles exceed the fixed capacity of %d\n",
                     (long long)n_tris, RT_NOALLOC_MAX_TRIS);
        return RT_ERR_TOO_LARGE;
    }
    if (n_tris == 0) return RT_OK;
    // an error the caller's own CUDA work left pending is theirs: report it without clearing
    // it, rather than taking it for a failure of the launches below
    if (cudaPeekAtLastError() != cudaSuccess) return RT_ERR_CUDA;
    void *base = nullptr;
    if (cudaGetSymbolAddress(&base, g_noalloc_scratch) != cudaSuccess || !base) {
        cudaGetLastError();   // the failed lookup's own error
        return RT_ERR_CUDA;
    }
    const int n = (int)n_tris;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    char *p = (char *)base;
    Scratch sc{};
    sc.box = (unsigned *)p;
    float *obj_pos = (float *)(p + 256);
    sc.centroid = (float4 *)(p + 512);
    int *tri_obj = (int *)(p + 512 + 16 * kNoAllocN);
    sc.codes[1] = (unsigned *)(p + 512 + 20 * kNoAllocN);
    sc.idx[1] = (unsigned *)(p + 512 + 24 * kNoAllocN);
    sc.hist = (unsigned *)(p + 512 + 28 * kNoAllocN);
    sc.part = (unsigned *)(p + 512 + 28 * kNoAllocN + 1024 * kNoAllocTiles);
    sc.codes[0] = d_codes;   // the caller's outputs are the other sort buffer: 4 passes end there
    sc.idx[0] = d_perm;
    // the array keeps the previous call's bytes: zero the object table this call reads
    if (cudaMemsetAsync(obj_pos, 0, 256, s) != cudaSuccess || cudaMemsetAsync(tri_obj, 0, 4 * (size_t)n, s) != cudaSuccess)
        return RT_ERR_CUDA;
    LbvhInput in{};
    in.tri_p = d_tri_p;
    in.tri_obj = tri_obj;
    in.obj_pos = obj_pos;
    in.n = n;
    if (morton_and_sort(in, sc, s) != cudaSuccess) return RT_ERR_CUDA;
    return RT_OK;
}
