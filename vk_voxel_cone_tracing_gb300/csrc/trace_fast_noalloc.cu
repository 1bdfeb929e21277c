// trace_fast_noalloc.cu -- vct_cone_trace_fast_noalloc: the fast cone tracer
// for callers that cannot allocate device memory.
//
// Who cannot allocate: renderers and plugin hosts that reserve every byte of
// GPU memory up front and hand it out through their own allocator, and
// real-time frame loops that must not call cudaMalloc / cudaFree (both can
// synchronise the device and stall a frame) or run where allocation is
// forbidden.  Such a caller still owns its samples and output buffers but
// has nowhere to put the sort keys, visiting orders and radix-sort temporary
// storage that vct_cone_trace_fast needs as scratch.
//
// This entry point keeps that scratch in a file-scope device array of
// VCT_NOALLOC_SCRATCH_BYTES.  The array is part of this translation unit's
// device module.  Under lazy module loading (CUDA_MODULE_LOADING=LAZY, the
// runtime's default) that module -- and with it the 48 MiB -- is committed on
// a device the first time this entry point runs there; with eager loading it
// is committed when the library's modules load.  Either way the device keeps
// it until the process exits, and no call ever runs cudaMalloc.  A host that
// reserves (nearly) all device memory for its own allocator must therefore
// make one call on each device before it makes that reservation, and before
// any stream capture.
//
// Host code cannot use the array's name as a device address, so every call
// looks the address up with cudaGetSymbolAddress on the current device (a
// table lookup once the module is loaded); nothing is cached across calls,
// so a context torn down and re-created (cudaDeviceReset) gets the new
// module's address.  All calls share the one array and it keeps the
// previous call's contents: the tracer clears what must start at zero (its
// specular counter) on every call, and calls whose GPU work overlaps -- on
// two streams, or from two host threads -- race on the array and must be
// serialised by the caller.
#include "common.cuh"

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[VCT_NOALLOC_SCRATCH_BYTES];

}  // namespace

extern "C" int vct_cone_trace_fast_noalloc(const vct_cone_tracing_desc* desc, const vct_cam_matrix* cam,
                                           vct_texture radiance, const vct_shadow_map* shadow,
                                           const vct_directional_light_desc* light,
                                           const vct_directional_light_shadow_desc* light_shadow,
                                           const vct_surface_sample* samples, int64_t sample_count,
                                           float* diffuse_out, float* specular_out, unsigned long long* cone_steps,
                                           void* stream) {
    VCT_CHECK_ARG(sample_count >= 0 && sample_count <= VCT_NOALLOC_MAX_SAMPLES,
                  "vct_cone_trace_fast_noalloc: sample count exceeds VCT_NOALLOC_MAX_SAMPLES (1048576); "
                  "use vct_cone_trace_fast with caller-provided scratch");
    const int64_t need = vct_cone_trace_fast_scratch_bytes(sample_count);
    if (need < 0 || need > (int64_t)VCT_NOALLOC_SCRATCH_BYTES)
        return vct::fail(VCT_E_BAD_ARG, "vct_cone_trace_fast_noalloc: the static scratch array is too small for "
                                        "this sample count");
    // the address on the current device, looked up with that device current
    void* scratch = nullptr;
    VCT_CUDA_TRY(cudaGetSymbolAddress(&scratch, g_noalloc_scratch));
    return vct_cone_trace_fast(desc, cam, radiance, shadow, light, light_shadow, samples, sample_count, diffuse_out,
                               specular_out, cone_steps, scratch, (size_t)VCT_NOALLOC_SCRATCH_BYTES, stream);
}
