// mip_pairs.cuh -- the front-to-back pairs of the anisotropic 2x2x2 mips
// (opacityDownSample.comp / radianceDownSample.comp): for face f (0/1: +x/-x,
// 2/3: +y/-y, 4/5: +z/-z) the four pairs (front, back) of child indices
// i = x | y << 1 | z << 2 along the face's axis, front first for the even
// face.  A constexpr function rather than a table in constant memory: with
// the face and pair loops unrolled every index is a compile-time constant, so
// a thread's eight children stay in registers (a table read made the index
// dynamic and put the children array in local memory).
#pragma once

namespace vct {

__host__ __device__ constexpr int ds_pair(int f, int k, int j) {
    // the k-th child with the face axis's bit clear, then j (flipped on odd faces) on that bit
    return (f >> 1) == 0 ? ((k << 1) | ((j ^ (f & 1)) & 1))
           : (f >> 1) == 1 ? ((k & 1) | ((k >> 1) << 2) | (((j ^ (f & 1)) & 1) << 1))
                           : (k | (((j ^ (f & 1)) & 1) << 2));
}

static_assert(ds_pair(0, 3, 0) == 6 && ds_pair(0, 3, 1) == 7 && ds_pair(1, 0, 0) == 1 && ds_pair(1, 0, 1) == 0,
              "x pairs");
static_assert(ds_pair(2, 2, 0) == 4 && ds_pair(2, 2, 1) == 6 && ds_pair(3, 1, 0) == 3 && ds_pair(3, 1, 1) == 1,
              "y pairs");
static_assert(ds_pair(4, 3, 0) == 3 && ds_pair(4, 3, 1) == 7 && ds_pair(5, 2, 0) == 6 && ds_pair(5, 2, 1) == 2,
              "z pairs");

}  // namespace vct
