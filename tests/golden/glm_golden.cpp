// glm_golden.cpp -- golden-vector generator (see make_golden.py).
//
// Evaluates, with the reference's vendored glm and its defines, the host-side
// math of the path: VoxelizationPass::createVoxelClipmap/calculateChangeDelta
// (VFS/RenderPass/Clipmap/VoxelizationPass.cpp:335-357, 438-448) fed by
// Application::updateClipRegionBoundingBox (VFS/Application.cpp:116-128),
// Voxelizer::setViewProjection (VFS/RenderPass/Clipmap/Voxelizer.cpp:394-423),
// DirectionalLight::setTransform (VFS/DirectionalLight.cpp:21-47),
// Camera::updateCamera (VFS/Camera.cpp:110-117) and the glTF node matrices
// (VFS/Util/GLTFLoader.cpp:399-431, VFS/GLTFScene.cpp:398-412).  The
// calls below are written here from those functions' arguments; nothing of
// the reference is compiled.  Prints JSON with every float as its bit pattern.
#define GLM_FORCE_SIZE_T_LENGTH
#define GLM_FORCE_DEPTH_ZERO_TO_ONE
#define GLM_FORCE_LEFT_HANDED
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <glm/gtc/quaternion.hpp>

static uint32_t bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

static void print_mat(const glm::mat4& m) {
    std::printf("[");
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) std::printf("%u%s", bits(m[c][r]), (c == 3 && r == 3) ? "" : ",");
    std::printf("]");
}

struct Region {
    glm::ivec3 minCorner;
    glm::uvec3 extent;
    float voxelSize;
};

int main() {
    const float cams[][3] = {{0.f, 0.f, 0.f}, {1.3f, 2.7f, -5.1f}, {-40.2f, 3.3f, 17.9f}, {0.37f, -0.51f, 8.9f}};
    const uint32_t resolutions[] = {64, 128, 256};
    const int32_t minChange[6] = {2, 2, 2, 2, 2, 1};
    std::printf("{\"regions\":[");
    bool first = true;
    for (auto& cam : cams)
        for (uint32_t R : resolutions) {
            Region regs[6];
            for (int l = 0; l < 6; ++l) {
                const uint32_t half = R >> 1;
                regs[l].minCorner = -glm::ivec3(half);
                regs[l].extent = glm::uvec3(R, R, R);
                regs[l].voxelSize = (16u * (1u << l)) / static_cast<float>(R);
                glm::vec3 center(cam[0], cam[1], cam[2]);
                const float halfSize = static_cast<float>((16u >> 1) * (1u << l));
                glm::vec3 bbMin = center - halfSize;
                glm::vec3 deltaW = bbMin - (glm::vec3(regs[l].minCorner) * regs[l].voxelSize);
                const float minChangeW = regs[l].voxelSize * minChange[l];
                glm::ivec3 delta = glm::ivec3(glm::trunc(deltaW / minChangeW)) * minChange[l];
                regs[l].minCorner += delta;
            }
            for (int l = 0; l < 6; ++l) {
                const Region& region = regs[l];
                Region ext = region;
                ext.extent = ext.extent + 2u;
                ext.minCorner -= 1;
                const glm::vec3 regionGlobal = glm::vec3(ext.extent) * ext.voxelSize;
                const glm::vec3 minCornerGlobal = glm::vec3(ext.minCorner) * ext.voxelSize;
                const glm::vec3 eye = minCornerGlobal + glm::vec3(0.0f, 0.0f, regionGlobal.z);
                glm::mat4 vp[3];
                vp[0] = glm::ortho(-regionGlobal.z, regionGlobal.z, -regionGlobal.y, regionGlobal.y, 0.1f, regionGlobal.x) *
                        glm::lookAt(eye, eye + glm::vec3(1.0f, 0.0f, 0.0f), glm::vec3(0.0f, 1.0f, 0.0f));
                vp[1] = glm::ortho(-regionGlobal.x, regionGlobal.x, -regionGlobal.z, regionGlobal.z, 0.1f, regionGlobal.y) *
                        glm::lookAt(eye, eye + glm::vec3(0.0f, 1.0f, 0.0f), glm::vec3(0.0f, 0.0f, -1.0f));
                vp[2] = glm::ortho(-regionGlobal.x, regionGlobal.x, -regionGlobal.y, regionGlobal.y, 0.1f, regionGlobal.z) *
                        glm::lookAt(minCornerGlobal, minCornerGlobal + glm::vec3(0.0f, 0.0f, 1.0f), glm::vec3(0.0f, 1.0f, 0.0f));
                std::printf("%s{\"cam\":[%u,%u,%u],\"R\":%u,\"level\":%d,\"min_corner\":[%d,%d,%d],\"voxel_size\":%u,\"view_proj\":[",
                            first ? "" : ",", bits(cam[0]), bits(cam[1]), bits(cam[2]), R, l, region.minCorner.x,
                            region.minCorner.y, region.minCorner.z, bits(region.voxelSize));
                first = false;
                for (int i = 0; i < 3; ++i) {
                    print_mat(vp[i]);
                    if (i < 2) std::printf(",");
                }
                std::printf("]}");
            }
        }
    std::printf("],\"lights\":[");
    const float lights[][6] = {{0.f, 30.f, -5.3f, 0.f, -1.f, 0.2f}, {0.f, 20.f, 0.f, 0.3f, -1.f, 0.2f},
                               {4.2f, 14.f, -4.0f, 0.3f, -1.f, 0.2f}};
    first = true;
    for (auto& L : lights) {
        glm::vec3 origin(L[0], L[1], L[2]);
        glm::vec3 dir = glm::normalize(glm::vec3(L[3], L[4], L[5]));
        glm::mat4 view = glm::lookAt(origin, origin + dir, glm::vec3(0.0f, 1.0f, 0.0f));
        glm::mat4 proj = glm::ortho(-16.0f, 16.0f, -16.0f, 16.0f, 0.1f, 30.0f);
        std::printf("%s{\"origin\":[%u,%u,%u],\"direction\":[%u,%u,%u],\"view\":", first ? "" : ",", bits(L[0]),
                    bits(L[1]), bits(L[2]), bits(L[3]), bits(L[4]), bits(L[5]));
        first = false;
        print_mat(view);
        std::printf(",\"proj\":");
        print_mat(proj);
        std::printf("}");
    }
    // Camera::updateCamera (VFS/Camera.cpp:110-117)
    std::printf("],\"cameras\":[");
    const float cams2[][11] = {{0.f, 2.f, -5.f, 0.f, 0.f, 1.f, 0.f, 1.f, 0.f, 60.f, 1.7777778f},
                               {1.3f, 2.7f, -5.1f, 0.3f, -0.2f, 0.93f, 0.f, 1.f, 0.f, 60.f, 1.5f},
                               {-4.f, 1.5f, 3.f, 0.8f, 0.1f, -0.59f, 0.f, 1.f, 0.f, 45.f, 1.0f},
                               {0.37f, 6.1f, 0.2f, 0.05f, -0.99f, 0.1f, 0.f, 1.f, 0.f, 75.f, 1.25f}};
    first = true;
    for (auto& c : cams2) {
        const glm::vec3 pos(c[0], c[1], c[2]), dir(c[3], c[4], c[5]), up(c[6], c[7], c[8]);
        const glm::mat4 view = glm::lookAt(pos, pos + dir, up);
        const glm::mat4 proj = glm::perspective(glm::radians(c[9]), c[10], 0.01f, 5000.0f);
        std::printf("%s{\"in\":[", first ? "" : ",");
        first = false;
        for (int i = 0; i < 11; ++i) std::printf("%u%s", bits(c[i]), i == 10 ? "" : ",");
        std::printf("],\"view_proj\":");
        print_mat(proj * view);
        std::printf(",\"view_proj_inv\":");
        print_mat(glm::inverse(view) * glm::inverse(proj));
        std::printf(",\"view\":");
        print_mat(view);
        std::printf(",\"proj\":");
        print_mat(proj);
        std::printf(",\"view_inv\":");
        print_mat(glm::inverse(view));
        std::printf(",\"proj_inv\":");
        print_mat(glm::inverse(proj));
        std::printf("}");
    }
    // GLTFLoader::processNode / GetLocalMatrix (VFS/Util/GLTFLoader.cpp:399-431,511-517) and
    // GLTFScene::uploadMatrixBuffer (VFS/GLTFScene.cpp:398-412): a chain of three nodes
    std::printf("],\"nodes\":[");
    // translation xyz, rotation quaternion xyzw (glTF order), scale xyz
    const float trs[][10] = {{1.5f, -2.0f, 0.25f, 0.0f, 0.38268343f, 0.0f, 0.92387953f, 2.0f, 2.0f, 2.0f},
                             {0.0f, 3.0f, -1.0f, 0.1f, 0.2f, 0.3f, 0.9273618f, 1.0f, 0.5f, 1.5f},
                             {-4.0f, 0.5f, 7.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.75f, 0.75f, 0.75f}};
    glm::mat4 parent(1.0f);
    first = true;
    for (auto& n : trs) {
        const glm::quat q(n[6], n[3], n[4], n[5]);  // glm::quat(w, x, y, z)
        const glm::mat4 local = glm::translate(glm::mat4(1.0f), glm::vec3(n[0], n[1], n[2])) * glm::mat4_cast(q) *
                                glm::scale(glm::mat4(1.0f), glm::vec3(n[7], n[8], n[9])) * glm::mat4(1.0f);
        const glm::mat4 world = parent * local;
        std::printf("%s{\"trs\":[", first ? "" : ",");
        first = false;
        for (int i = 0; i < 10; ++i) std::printf("%u%s", bits(n[i]), i == 9 ? "" : ",");
        std::printf("],\"local\":");
        print_mat(local);
        std::printf(",\"world\":");
        print_mat(world);
        std::printf(",\"it_world\":");
        print_mat(glm::transpose(glm::inverse(world)));
        std::printf("}");
        parent = world;
    }
    std::printf("]}\n");
    return 0;
}
