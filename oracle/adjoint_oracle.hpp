// adjoint_oracle.hpp -- TEST INFRASTRUCTURE ONLY.
//
// FP64 reference gradients of the differentiable form, derived by reverse-mode
// automatic differentiation (ad_tape.hpp) of the oracle's own restatement:
//   * cone_trace_grad_f4: d/d(float atlas) of sum_i gd_i . diffuse_i +
//     gs_i . specular_i, where diffuse / specular are trace_sample's outputs
//     (voxelConeTracing.frag:143-294; trace_cone :341-392) over a float RGBA
//     atlas read through texture3d with FP64 arithmetic -- the function
//     vcto_cone_trace_f4 evaluates;
//   * downsample_chain_grad_f4: the adjoint of the radiance / opacity mips
//     (radianceDownSample.comp:28-139 with the opacity shader's lerpFactor
//     scoping, opacityDownSample.comp:28-138), levels `first`..5 in order, on
//     FP64 storage.
// Neither shares code with the GPU adjoint (trace_grad.cu, the mip adjoint in
// clipmap_passes.cu); both differentiate exactly what the FP64 oracle runs.
#pragma once

#include <vector>

#include "clipmap_oracle.hpp"

namespace vcto {

// Texel fetch whose values are leaves of the tape: scalar k = 4 * texel + c.
struct Float4VarFetch {
    const float* atlas;
    Atlas A;
    V4<ad::Var> operator()(int x, int y, int z) const {
        const int64_t t = A.index(x, y, z);
        const float* p = atlas + 4 * t;
        return V4<ad::Var>(ad::Var::leaf(p[0], 4 * t), ad::Var::leaf(p[1], 4 * t + 1), ad::Var::leaf(p[2], 4 * t + 2),
                           ad::Var::leaf(p[3], 4 * t + 3));
    }
};

// grad (4 doubles per texel, accumulated into) += d/d(atlas) of
// sum_{i in [begin, end)} gd[4i..4i+3] . diffuse_i + gs[4i..4i+3] . specular_i.
// Samples are split over threads, each with its own tape and gradient.
inline void cone_trace_grad_f4(const TraceDesc& desc, const float eye[3], const float* atlas4, int R,
                               const float* shadow, int sw, int sh, const ShadowDesc& sd, const LightDesc& light,
                               const SurfaceSample* samples, int64_t begin, int64_t end, const float* gd,
                               const float* gs, double* grad) {
    Atlas A(R);
    const int64_t n_scalars = 4 * A.texels();
#pragma omp parallel
    {
        std::vector<double> local(n_scalars, 0.0);
        std::vector<double> adj;
#pragma omp for schedule(dynamic, 4)
        for (int64_t i = begin; i < end; ++i) {
            ad::tape().clear();
            Float4VarFetch f{atlas4, A};
            ClipmapTracer<ad::Var, Float4VarFetch> tr{desc, f, A};
            ad::Var d[4], s[4];
            if (!trace_sample<ad::Var>(tr, eye, shadow, sw, sh, sd, light, samples[i], d, s)) continue;
            adj.assign(ad::tape().size(), 0.0);
            for (int c = 0; c < 4; ++c) {
                ad::seed(adj, local.data(), d[c], gd[4 * i + c]);
                ad::seed(adj, local.data(), s[c], gs[4 * i + c]);
            }
            ad::backward(adj, local.data());
        }
        ad::tape().clear();
#pragma omp critical
        for (int64_t k = 0; k < n_scalars; ++k) grad[k] += local[k];
    }
}

// Texel store of ad::Var values (FP64, no rounding); serial (one tape).
struct VarStore {
    std::vector<ad::Var>* vals;
    static constexpr bool kParallel = false;
    template <class T> V4<T> load(int64_t t) const {
        const ad::Var* p = vals->data() + 4 * t;
        return V4<T>(p[0], p[1], p[2], p[3]);
    }
    template <class T> void put(int64_t t, int c, T v) { (*vals)[4 * t + c] = v; }
};

// G (4 doubles per texel) enters holding dL/d(atlas after levels first..5)
// and leaves holding dL/d(atlas before them).  prev_min[l - 1] is the level
// l - 1 region's min corner (the DownSampleDesc of level l).
inline void downsample_chain_grad_f4(const float* atlas4, int R, const int prev_min[5][3], int first, int band,
                                     int mode, double* G) {
    Atlas A(R);
    const int64_t n = 4 * A.texels();
    std::vector<ad::Var> vals(n);
    for (int64_t k = 0; k < n; ++k) vals[k] = ad::Var::leaf(atlas4[k], k);
    ad::tape().clear();
    VarStore st{&vals};
    for (int level = first; level <= 5; ++level)
        downsample_f4_on<ad::Var>(st, R, prev_min[level - 1], level, band, mode);
    std::vector<double> adj(ad::tape().size(), 0.0);
    std::vector<double> out(n, 0.0);
    for (int64_t k = 0; k < n; ++k) ad::seed(adj, out.data(), vals[k], G[k]);
    ad::backward(adj, out.data());
    ad::tape().clear();
    for (int64_t k = 0; k < n; ++k) G[k] = out[k];
}

}  // namespace vcto
