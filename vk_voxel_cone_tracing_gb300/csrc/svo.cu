// svo.cu -- sparse voxel octree build over a uint2 node pool
// (OctreeBuilder::cmdBuild, VFS/RenderPass/Octree/OctreeBuilder.cpp:205-345).
//
// Node: x = MSB flag | child block index (8 children), y = RGBA8 colour.
// Per level: init the window, flag (every fragment descends from the root and
// sets its node's MSB; atomicOr, order-free), allocate a child block for every
// flagged node of the window.  VCT_SVO_DETERMINISTIC allocates by an exclusive
// scan over the window's flags -- the canonical breadth-first order -- and
// folds leaf colours in fragment order (stable sort by leaf, sequential CAS
// body); VCT_SVO_ATOMIC runs the reference's racy atomicAdd allocation and CAS
// loops.  Mips (octreeNodeMipmapWrite.comp) are computed per node: the shader
// writes, for each power-of-two target level t <= 2^(L-1), the flagged nodes
// at resolution t; a per-node pass over those windows gives the same values
// without the shader's per-fragment redundancy.
// Compiled with -fmad=false.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "common.cuh"

namespace vct {

__device__ inline uint3 frag_pos(uint2 f) {
    return make_uint3((f.x & 0xfffu) >> 1, ((f.x >> 12) & 0xfffu) >> 1,
                      (((f.x >> 24) & 0xffu) | ((f.y >> 20) & 0xf00u)) >> 1);
}

// do { ... } while (cur != 0 && res > limit), as in the node shaders.
__device__ inline uint32_t descend(const uint2* __restrict__ pool, uint3 p, uint32_t res, uint32_t limit,
                                   uint32_t& res_out) {
    uint32_t idx = 0, cur = 0;
    do {
        res >>= 1;
        const uint32_t cx = p.x >= res, cy = p.y >= res, cz = p.z >= res;
        idx = cur + (cz | (cx << 1) | (cy << 2));
        cur = pool[idx].x & 0x7fffffffu;
        p.x -= cx * res;
        p.y -= cy * res;
        p.z -= cz * res;
    } while (cur != 0u && res > limit);
    res_out = res;
    return idx;
}

__global__ void k_init(uint2* pool, uint64_t begin, uint64_t num) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < num; i += (uint64_t)gridDim.x * blockDim.x)
        pool[begin + i] = make_uint2(0u, 0u);
}

// Child slot a fragment takes at descent step k (resolution 2^(L-1-k)).  The
// node shaders descend from the root subtracting the resolution where
// pos >= resolution; for the halved position p <= 2^(L-1) that is: step 0
// takes the upper child only when p == 2^(L-1) (and leaves p = 0), later
// steps take bit (L-1-k) of the remaining p.  So the node a fragment reaches
// at depth i is the depth-(i-1) node's child block plus slot(i-1): one step
// per level from a per-fragment cursor instead of a descent from the root.
__device__ inline uint32_t slot_at(uint3 p, int L, int k) {
    const uint32_t top = 1u << (L - 1);
    if (k == 0) return (p.z >= top ? 1u : 0u) | (p.x >= top ? 2u : 0u) | (p.y >= top ? 4u : 0u);
    const uint3 q = make_uint3(p.x >= top ? p.x - top : p.x, p.y >= top ? p.y - top : p.y, p.z >= top ? p.z - top : p.z);
    const int b = L - 1 - k;
    return ((q.z >> b) & 1u) | (((q.x >> b) & 1u) << 1) | (((q.y >> b) & 1u) << 2);
}

// octreeNodeFlag.comp for level i through the cursor; the flag is written
// only if not yet set (the shader's racy |= is idempotent either way).
__global__ void k_flag_level(uint2* pool, const uint2* __restrict__ frags, int64_t F, int L, int level,
                             uint32_t* __restrict__ cursor) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < F; i += (int64_t)gridDim.x * blockDim.x) {
        const uint3 p = frag_pos(__ldg(frags + i));
        const uint32_t slot = slot_at(p, L, level - 1);
        const uint32_t node = level == 1 ? slot : (pool[cursor[i]].x & 0x7fffffffu) + slot;
        cursor[i] = node;
        if (!(pool[node].x & 0x80000000u)) atomicOr(&pool[node].x, 0x80000000u);
    }
}

__global__ void k_window_flags(const uint2* __restrict__ pool, uint64_t begin, uint64_t num, uint32_t* __restrict__ f) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < num; i += (uint64_t)gridDim.x * blockDim.x)
        f[i] = pool[begin + i].x >> 31;
}

__global__ void k_alloc_scan(uint2* pool, uint64_t begin, uint64_t num, const uint32_t* __restrict__ rank,
                             uint64_t counter) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < num; i += (uint64_t)gridDim.x * blockDim.x) {
        uint2 n = pool[begin + i];
        if (n.x & 0x80000000u) pool[begin + i] = make_uint2((uint32_t)((counter + rank[i] + 1) << 3) | 0x80000000u, 0u);
    }
}

// octreeNodeAlloc.comp with a warp-aggregated counter increment (one atomicAdd per warp).
__global__ void k_alloc_atomic(uint2* pool, uint64_t begin, uint64_t num, unsigned int* counter) {
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); base < num; base += stride) {
        const uint64_t i = base + lane;
        const bool flagged = i < num && (pool[begin + i].x & 0x80000000u);
        const unsigned m = __ballot_sync(0xffffffffu, flagged);
        unsigned wbase = 0;
        if (lane == 0 && m) wbase = atomicAdd(counter, (unsigned)__popc(m));
        wbase = __shfl_sync(0xffffffffu, wbase, 0);
        if (flagged) {
            const unsigned c = wbase + __popc(m & ((1u << lane) - 1u));
            pool[begin + i] = make_uint2(((c + 1u) << 3) | 0x80000000u, 0u);
        }
    }
}

__device__ inline uint32_t conv_u8x4(float x, float y, float z, float w) {
    return (((uint32_t)w & 0xffu) << 24) | (((uint32_t)z & 0xffu) << 16) | (((uint32_t)y & 0xffu) << 8) |
           ((uint32_t)x & 0xffu);
}

__device__ inline uint32_t avg_fold(uint32_t cur, uint32_t v) {
    const float vr = (float)(v & 0xffu), vg = (float)((v >> 8) & 0xffu), vb = (float)((v >> 16) & 0xffu),
                va = (float)(v >> 24);
    if (cur == 0u) return conv_u8x4(vr, vg, vb, va);
    float rx = (float)(cur & 0xffu), ry = (float)((cur >> 8) & 0xffu), rz = (float)((cur >> 16) & 0xffu),
          rw = (float)(cur >> 24);
    rx = rx * rw;
    ry = ry * rw;
    rz = rz * rw;
    float cx = rx + vr, cy = ry + vg, cz = rz + vb, cw = rw + va;
    cx = cx / cw;
    cy = cy / cw;
    cz = cz / cw;
    return conv_u8x4(cx, cy, cz, cw);
}

// Leaf of each fragment: its cursor after the last level (the depth-L node
// octreeNodeLeafWrite.comp's descent reaches at resolution 1).
__global__ void k_leaf_keys(const uint32_t* __restrict__ cursor, int64_t F, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < F; i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = cursor[i];
        vals[i] = (uint32_t)i;
    }
}

// Boundaries of the leaf runs in the sorted keys over positions [0, n]: every
// position whose key differs from its predecessor, plus 0 and n.
struct LeafRunHead {
    const uint32_t* keys;
    uint32_t n;
    __device__ bool operator()(uint32_t i) const { return i == 0 || i == n || keys[i - 1] != keys[i]; }
};

// Sequential fold of each leaf's fragments in fragment order (the stable sort
// keeps it), one thread per leaf run.
__global__ void __launch_bounds__(256) k_leaf_fold(uint2* pool, const uint2* __restrict__ frags,
                                                   const uint32_t* __restrict__ keys, const uint32_t* __restrict__ order,
                                                   const uint32_t* __restrict__ heads,
                                                   const uint32_t* __restrict__ nheads) {
    const uint32_t nruns = *nheads - 1u;
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nruns; h += gridDim.x * blockDim.x) {
        const uint32_t s = heads[h], e = heads[h + 1];
        const uint32_t key = keys[s];
        uint32_t cell = pool[key].y;
        // the fold is a serial chain; fetch four fragments ahead of it
        for (uint32_t j = s; j < e; j += 4) {
            uint32_t v4[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j + u < e) v4[u] = __ldg(&frags[order[j + u]].y) & 0xfffffffu;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j + u < e) cell = avg_fold(cell, v4[u]);
        }
        pool[key].y = cell;
    }
}

__global__ void k_leaf_atomic(uint2* pool, const uint2* __restrict__ frags, int64_t F,
                              const uint32_t* __restrict__ cursor, int* err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < F; i += (int64_t)gridDim.x * blockDim.x) {
        const uint2 f = __ldg(frags + i);
        const uint32_t idx = cursor[i];
        const uint32_t v = f.y & 0xfffffffu;
        uint32_t prev = 0u, newv = avg_fold(0u, v), cur;
        int guard = 0;
        while ((cur = atomicCAS(&pool[idx].y, prev, newv)) != prev) {
            prev = cur;
            newv = avg_fold(cur, v);
            if (++guard > (1 << 20)) {
                atomicExch(err, 1);
                break;
            }
        }
    }
}

// Per-node mip of one window (octreeNodeMipmapWrite.comp:50-60): y = sum(child/8).
__global__ void k_mip_nodes(uint2* pool, uint64_t begin, uint64_t num) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < num; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 n = pool[begin + i];
        if (!(n.x & 0x80000000u)) continue;
        const uint32_t child = n.x & 0x7fffffffu;
        float s[4] = {0.f, 0.f, 0.f, 0.f};
        for (int j = 0; j < 8; ++j) {
            const uint32_t v = pool[child + j].y;
#pragma unroll
            for (int c = 0; c < 4; ++c) s[c] = s[c] + (float)((v >> (8 * c)) & 0xffu) / 8.0f;
        }
        pool[begin + i].y = conv_u8x4(s[0], s[1], s[2], s[3]);
    }
}

// Canonical relabelling, one level: new window nodes read their old node via new2old.
__global__ void k_canon_flags(const uint2* __restrict__ in, const uint32_t* __restrict__ new2old, uint64_t begin,
                              uint64_t num, uint32_t* __restrict__ f) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < num; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 n = in[new2old[begin + i]];
        f[i] = (n.x >> 31) && (n.x & 0x7fffffffu) ? 1u : 0u;
    }
}

__global__ void k_canon_write(const uint2* __restrict__ in, uint2* __restrict__ out, uint32_t* __restrict__ new2old,
                              uint64_t begin, uint64_t num, const uint32_t* __restrict__ rank, uint64_t counter) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < num; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 n = in[new2old[begin + i]];
        uint32_t x = n.x & 0x80000000u;
        const uint32_t oc = n.x & 0x7fffffffu;
        if ((n.x >> 31) && oc) {
            const uint32_t nc = (uint32_t)((counter + rank[i] + 1) << 3);
            x |= nc;
            for (int c = 0; c < 8; ++c) new2old[nc + c] = oc + c;
        }
        out[begin + i] = make_uint2(x, n.y);
    }
}

static int grid_n(uint64_t n, int block = 256) {
    uint64_t g = (n + block - 1) / block;
    return (int)(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}
static size_t a256s(size_t x) { return (x + 255) & ~size_t(255); }

// Exclusive scan of `num` 0/1 flags -> ranks; returns the number of ones (host).
static int scan_flags(const uint32_t* flags, uint32_t* rank, uint64_t num, void* tmp, size_t tmp_bytes,
                      uint32_t* d_tail, uint64_t* ones, cudaStream_t st) {
    size_t tb = tmp_bytes;
    VCT_CUDA_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, flags, rank, (int)num, st));
    uint32_t h[2];
    VCT_CUDA_TRY(cudaMemcpyAsync(&h[0], rank + (num - 1), 4, cudaMemcpyDeviceToHost, st));
    VCT_CUDA_TRY(cudaMemcpyAsync(&h[1], flags + (num - 1), 4, cudaMemcpyDeviceToHost, st));
    VCT_CUDA_TRY(cudaStreamSynchronize(st));
    (void)d_tail;
    *ones = (uint64_t)h[0] + h[1];
    return VCT_OK;
}

}  // namespace vct

using namespace vct;

extern "C" int64_t vct_svo_pool_capacity(int64_t F) {
    if (F < 0) return -1;
    int64_t n = F * 8;
    if (n < (int64_t)VCT_MIN_OCTREE_NODE_NUM) n = VCT_MIN_OCTREE_NODE_NUM;
    if (n > (int64_t)VCT_MAX_OCTREE_NODE_NUM) n = VCT_MAX_OCTREE_NODE_NUM;
    return n;
}

extern "C" int vct_svo_build(const uint32_t* fragments, int64_t F, int32_t L, uint32_t* pool_u32, int64_t capacity,
                             int32_t mode, int64_t* node_count, vct_workspace_s* ws, void* stream) {
    vct::NvtxRange nvtx_range("vct_svo_build");
    VCT_CHECK_ARG(node_count && ws, "vct_svo_build: null argument");
    VCT_CHECK_ARG(L >= 1 && L <= 11, "vct_svo_build: octree level must be 1..11");
    VCT_CHECK_ARG(F >= 0 && F < (1LL << 31), "vct_svo_build: fragment count out of range");
    VCT_CHECK_ARG(F == 0 || fragments, "vct_svo_build: null fragment list");
    VCT_CHECK_ARG(pool_u32 && capacity >= 8 && capacity < (1LL << 31), "vct_svo_build: bad node pool");
    VCT_CHECK_ARG(mode == VCT_SVO_DETERMINISTIC || mode == VCT_SVO_ATOMIC, "vct_svo_build: bad mode");
    *node_count = 0;
    cudaStream_t st = as_stream(stream);
    uint2* pool = reinterpret_cast<uint2*>(pool_u32);
    const uint2* frags = reinterpret_cast<const uint2*>(fragments);
    const uint32_t res = 1u << L;
    // workspace: flags, ranks (window sized: <= capacity), scan temp, counter, leaf sort buffers
    size_t scan_bytes = 0, sort_bytes = 0, select_bytes = 0;
    VCT_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)capacity));
    const int64_t Fs = F > 0 ? F : 1;
    VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                                 (uint32_t*)nullptr, (uint32_t*)nullptr, (int)Fs, 0, 32));
    VCT_CUDA_TRY(cub::DeviceSelect::If(nullptr, select_bytes, thrust::counting_iterator<uint32_t>(0u), (uint32_t*)nullptr,
                                       (uint32_t*)nullptr, (int64_t)Fs + 1, LeafRunHead{nullptr, (uint32_t)Fs}));
    if (select_bytes > sort_bytes) sort_bytes = select_bytes;
    const size_t cap_arr = a256s(4 * (size_t)capacity), f_arr = a256s(4 * (size_t)Fs + 4);
    const size_t need = 2 * cap_arr + a256s(scan_bytes) + 256 + 6 * f_arr + 256 + a256s(sort_bytes);
    int rc = workspace_reserve(ws, need);
    if (rc != VCT_OK) return rc;
    char* b = (char*)ws->ptr;
    uint32_t* flags = (uint32_t*)b;
    uint32_t* rank = (uint32_t*)(b + cap_arr);
    void* tmp = b + 2 * cap_arr;
    unsigned int* counter = (unsigned int*)(b + 2 * cap_arr + a256s(scan_bytes));
    char* fb = b + 2 * cap_arr + a256s(scan_bytes) + 256;
    uint32_t* kin = (uint32_t*)fb;
    uint32_t* kout = (uint32_t*)(fb + f_arr);
    uint32_t* vin = (uint32_t*)(fb + 2 * f_arr);
    uint32_t* vout = (uint32_t*)(fb + 3 * f_arr);
    uint32_t* cursor = (uint32_t*)(fb + 4 * f_arr);
    uint32_t* heads = (uint32_t*)(fb + 5 * f_arr);
    uint32_t* nheads = (uint32_t*)(fb + 6 * f_arr);
    void* stmp = fb + 6 * f_arr + 256;

    uint64_t begin = 0, num = 8, count = 0;
    uint64_t wbegin[12], wnum[12];
    if (mode == VCT_SVO_ATOMIC) VCT_CUDA_TRY(cudaMemsetAsync(counter, 0, 4, st));
    for (int i = 1; i <= L; ++i) {
        if (begin + num > (uint64_t)capacity) return fail(VCT_E_OVERFLOW, "vct_svo_build: node pool capacity exceeded");
        wbegin[i] = begin;
        wnum[i] = num;
        k_init<<<grid_n(num), 256, 0, st>>>(pool, begin, num);
        if (F) k_flag_level<<<grid_n(F), 256, 0, st>>>(pool, frags, F, L, i, cursor);
        VCT_LAUNCH_CHECK();
        if (i != L) {
            uint64_t ones = 0;
            if (mode == VCT_SVO_DETERMINISTIC) {
                k_window_flags<<<grid_n(num), 256, 0, st>>>(pool, begin, num, flags);
                VCT_LAUNCH_CHECK();
                rc = scan_flags(flags, rank, num, tmp, scan_bytes, nullptr, &ones, st);
                if (rc != VCT_OK) return rc;
                k_alloc_scan<<<grid_n(num), 256, 0, st>>>(pool, begin, num, rank, count);
                VCT_LAUNCH_CHECK();
                count += ones;
            } else {
                k_alloc_atomic<<<grid_n(num), 256, 0, st>>>(pool, begin, num, counter);
                VCT_LAUNCH_CHECK();
                uint32_t c;
                VCT_CUDA_TRY(cudaMemcpyAsync(&c, counter, 4, cudaMemcpyDeviceToHost, st));
                VCT_CUDA_TRY(cudaStreamSynchronize(st));
                count = c;
            }
            begin += num;  // octreeNodeModifyArg.comp
            num = count * 8 + 8 - begin;
        }
    }
    *node_count = (int64_t)(count * 8 + 8);
    // leaf colours
    if (F) {
        if (mode == VCT_SVO_DETERMINISTIC) {
            k_leaf_keys<<<grid_n(F), 256, 0, st>>>(cursor, F, kin, vin);
            VCT_LAUNCH_CHECK();
            // leaf indices are node indices < node_count: sort only those bits
            const int key_bits = 32 - __builtin_clz((unsigned)(*node_count - 1));
            size_t tb = sort_bytes;
            VCT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(stmp, tb, kin, kout, vin, vout, (int)F, 0, key_bits, st));
            tb = sort_bytes;
            VCT_CUDA_TRY(cub::DeviceSelect::If(stmp, tb, thrust::counting_iterator<uint32_t>(0u), heads, nheads,
                                               (int64_t)F + 1, LeafRunHead{kout, (uint32_t)F}, st));
            k_leaf_fold<<<grid_n(F), 256, 0, st>>>(pool, frags, kout, vout, heads, nheads);
            VCT_LAUNCH_CHECK();
        } else {
            int* err = (int*)flags;
            VCT_CUDA_TRY(cudaMemsetAsync(err, 0, 4, st));
            k_leaf_atomic<<<grid_n(F), 256, 0, st>>>(pool, frags, F, cursor, err);
            VCT_LAUNCH_CHECK();
            int herr = 0;
            VCT_CUDA_TRY(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
            VCT_CUDA_TRY(cudaStreamSynchronize(st));
            if (herr) return fail(VCT_E_TIMEOUT, "vct_svo_build: a CAS loop gave up after 2^20 retries");
        }
    }
    // mips: targets t = 2, 4, 8, ... <= L and <= 2^(L-1): the window at depth L - log2(t)
    for (int k = 1; (1 << k) <= L && k <= L - 1; ++k) {
        const int depth = L - k;
        if (F) k_mip_nodes<<<grid_n(wnum[depth]), 256, 0, st>>>(pool, wbegin[depth], wnum[depth]);
        VCT_LAUNCH_CHECK();
    }
    return VCT_OK;
}

extern "C" int vct_svo_canonicalize(const uint32_t* pool_in_u32, int64_t node_count, int32_t L, uint32_t* pool_out_u32,
                                    vct_workspace_s* ws, void* stream) {
    VCT_CHECK_ARG(pool_in_u32 && pool_out_u32 && ws && pool_in_u32 != pool_out_u32, "vct_svo_canonicalize: bad argument");
    VCT_CHECK_ARG(L >= 1 && L <= 11 && node_count >= 8 && node_count < (1LL << 31), "vct_svo_canonicalize: bad size");
    cudaStream_t st = as_stream(stream);
    const uint2* in = reinterpret_cast<const uint2*>(pool_in_u32);
    uint2* out = reinterpret_cast<uint2*>(pool_out_u32);
    size_t scan_bytes = 0;
    VCT_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)node_count));
    const size_t arr = a256s(4 * (size_t)node_count);
    int rc = workspace_reserve(ws, 3 * arr + a256s(scan_bytes));
    if (rc != VCT_OK) return rc;
    char* b = (char*)ws->ptr;
    uint32_t* new2old = (uint32_t*)b;
    uint32_t* flags = (uint32_t*)(b + arr);
    uint32_t* rank = (uint32_t*)(b + 2 * arr);
    void* tmp = b + 3 * arr;
    const uint32_t ident[8] = {0, 1, 2, 3, 4, 5, 6, 7};
    VCT_CUDA_TRY(cudaMemcpyAsync(new2old, ident, sizeof(ident), cudaMemcpyHostToDevice, st));
    uint64_t begin = 0, num = 8, count = 0;
    for (int i = 1; i <= L && num > 0; ++i) {
        if (begin + num > (uint64_t)node_count) return fail(VCT_E_BAD_ARG, "vct_svo_canonicalize: pool is not a complete build");
        k_canon_flags<<<grid_n(num), 256, 0, st>>>(in, new2old, begin, num, flags);
        VCT_LAUNCH_CHECK();
        uint64_t ones = 0;
        rc = scan_flags(flags, rank, num, tmp, scan_bytes, nullptr, &ones, st);
        if (rc != VCT_OK) return rc;
        k_canon_write<<<grid_n(num), 256, 0, st>>>(in, out, new2old, begin, num, rank, count);
        VCT_LAUNCH_CHECK();
        count += ones;
        begin += num;
        num = count * 8 + 8 - begin;
    }
    return VCT_OK;
}
