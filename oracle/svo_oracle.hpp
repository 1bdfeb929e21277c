// svo_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the sparse-voxel-octree build of the reference
// (OctreeBuilder::cmdBuild, VFS/RenderPass/Octree/OctreeBuilder.cpp:205-345)
// and its six compute shaders:
//   octreeNodeInit.comp:15-24, octreeNodeFlag.comp:20-47,
//   octreeNodeAlloc.comp:20-34, octreeNodeModifyArg.comp:22-27,
//   octreeNodeLeafWrite.comp:26-89, octreeNodeMipmapWrite.comp:26-96.
// Node pool: uint2 per node, x = MSB flag | child block index, y = RGBA8.
// Node allocation is the sequential order of the atomic counter when the
// flagged nodes of a window are visited in index order (the canonical
// breadth-first order); the reference's racy allocation differs from it only by
// a relabelling of child blocks.
#pragma once

#include <cstdint>
#include <vector>

#include "raster_oracle.hpp"

namespace vcto {

struct SvoPos {
    uint32_t x, y, z;
};

// Packed fragment -> position, halved (the shaders' ">> 1", octreeNodeFlag.comp:28-32).
inline SvoPos svo_frag_pos(const uint32_t* f) {
    SvoPos p;
    p.x = (f[0] & 0xfffu) >> 1;
    p.y = ((f[0] >> 12) & 0xfffu) >> 1;
    p.z = (((f[0] >> 24) & 0xffu) | ((f[1] >> 20) & 0xf00u)) >> 1;
    return p;
}

// The shared descent: returns idx; `res_out` receives the final resolution.
// stop(res) decides whether to continue after a step: the loop runs
// "do { ... } while (cur != 0 && res > limit)".
inline uint32_t svo_descend(const uint32_t* pool, SvoPos p, uint32_t resolution, uint32_t limit, uint32_t& res_out) {
    uint32_t idx = 0, cur = 0;
    do {
        resolution >>= 1;
        const uint32_t cx = p.x >= resolution, cy = p.y >= resolution, cz = p.z >= resolution;
        idx = cur + (cz | (cx << 1) | (cy << 2));
        cur = pool[2 * (uint64_t)idx] & 0x7fffffffu;
        p.x -= cx * resolution;
        p.y -= cy * resolution;
        p.z -= cz * resolution;
    } while (cur != 0u && resolution > limit);
    res_out = resolution;
    return idx;
}

// Top-down subdivision (cmdNodeSubdivision).  Returns 0, or -1 if the pool
// capacity would be exceeded (the reference writes out of bounds there).
inline int svo_subdivide(const uint32_t* frags, int64_t F, int octree_level, uint32_t* pool, int64_t capacity,
                         int64_t* node_count) {
    const uint32_t res = 1u << octree_level;
    uint64_t begin = 0, num = 8, counter = 0;
    if (capacity < 8) return -1;
    for (int i = 1; i <= octree_level; ++i) {
        if (begin + num > (uint64_t)capacity) return -1;
        for (uint64_t k = begin; k < begin + num; ++k) pool[2 * k] = pool[2 * k + 1] = 0u;  // Init
        for (int64_t f = 0; f < F; ++f) {                                                   // Flag
            uint32_t r;
            uint32_t idx = svo_descend(pool, svo_frag_pos(frags + 2 * f), res, 1u, r);
            pool[2 * (uint64_t)idx] |= 0x80000000u;
        }
        if (i != octree_level) {
            for (uint64_t k = begin; k < begin + num; ++k) {  // Alloc
                if (pool[2 * k] & 0x80000000u) {
                    const uint64_t c = counter++;
                    pool[2 * k] = (uint32_t)((c + 1) << 3) | 0x80000000u;
                    pool[2 * k + 1] = 0u;
                }
            }
            begin += num;  // ModifyArg
            num = counter * 8 + 8 - begin;
        }
    }
    *node_count = (int64_t)(counter * 8 + 8);
    return 0;
}

// octreeNodeLeafWrite.comp: RGBA8 running average of the 28-bit fragment
// colour (alpha 15 per fragment, wrapping at 256) into each reached leaf.
inline void svo_leaf_write(const uint32_t* frags, int64_t F, int octree_level, uint32_t* pool) {
    const uint32_t res = 1u << octree_level;
    for (int64_t f = 0; f < F; ++f) {
        uint32_t r;
        uint32_t idx = svo_descend(pool, svo_frag_pos(frags + 2 * f), res, 1u, r);
        if (r == 1u) {
            const uint32_t v = frags[2 * f + 1] & 0xfffffffu;
            uint32_t& cell = pool[2 * (uint64_t)idx + 1];
            cell = rgba8_avg_fold(cell, (float)(v & 0xffu), (float)((v >> 8) & 0xffu), (float)((v >> 16) & 0xffu),
                                  (float)(v >> 24));
        }
    }
}

// octreeNodeMipmapWrite.comp for targetLevel = 2..L: the descent stops when
// resolution <= targetLevel and writes only if resolution == targetLevel, so
// only power-of-two target levels below the root resolution produce mips.
inline void svo_mip_write(const uint32_t* frags, int64_t F, int octree_level, uint32_t* pool) {
    const uint32_t res = 1u << octree_level;
    for (int target = 2; target <= octree_level; ++target) {
        for (int64_t f = 0; f < F; ++f) {
            uint32_t r;
            uint32_t idx = svo_descend(pool, svo_frag_pos(frags + 2 * f), res, (uint32_t)target, r);
            if (r == (uint32_t)target) {
                const uint32_t child = pool[2 * (uint64_t)idx] & 0x7fffffffu;
                float s[4] = {0.f, 0.f, 0.f, 0.f};
                for (int j = 0; j < 8; ++j) {
                    const uint32_t v = pool[2 * ((uint64_t)child + j) + 1];
                    for (int c = 0; c < 4; ++c) s[c] = s[c] + (float)((v >> (8 * c)) & 0xffu) / 8.0f;
                }
                pool[2 * (uint64_t)idx + 1] = (((uint32_t)s[3] & 0xffu) << 24) | (((uint32_t)s[2] & 0xffu) << 16) |
                                              (((uint32_t)s[1] & 0xffu) << 8) | ((uint32_t)s[0] & 0xffu);
            }
        }
    }
}

}  // namespace vcto
