// naive_path_host.cpp — a C++ caller of libzgl shaped like the reference's
// integrator layer, as INTEGRATION.md describes the drop-in.
//
// The reference's renderer drives `class Integrator` (src/core/Integrator.h:
// 25-52) and NaivePathIntegrator::renderOnePass / reset
// (src/integrator/NaivePath.cpp:77-115) against a scene from Scene::load.
// Here the same interface is a thin C++ class over the C ABI: init creates a
// ZGL integrator on the scene that zgl_scene_load_xml returned, renderOnePass
// forwards to zgl_integrator_render_pass, reset to zgl_integrator_reset,
// resultScale to zgl_integrator_result_scale, and the frame is read back
// from the integrator's running sum.  The GUI methods of the reference's
// interface have no work to do here.
//
// Usage: naive_path_host <scene.xml> <passes> <passes after reset> <max depth> <out.bin>
// out.bin: int32 W, int32 H, int32 spp, float resultScale, float[H][W][4] frame.
// Built and run by tests/test_cpp_host_gpu.py.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "zgl.h"

namespace {

struct RenderStatus {
    int width = 0, height = 0;
};

// The reference's Integrator interface, without its OpenGL frame texture.
class Integrator {
public:
    virtual ~Integrator() = default;
    virtual bool init(zgl_scene* scene, int width, int height) = 0;
    virtual bool renderOnePass() = 0;
    virtual bool reset(const RenderStatus& status) = 0;
    virtual float resultScale() const = 0;
    void setStatus(const RenderStatus& status) { mStatus = status; }
    void setShouldReset() { mShouldReset = true; }

protected:
    RenderStatus mStatus;
    bool mShouldReset = false;
};

bool ok(zgl_status st, const char* what) {
    if (st == ZGL_OK) return true;
    std::fprintf(stderr, "%s failed: %s\n", what, zgl_last_error());
    return false;
}

// NaivePathIntegrator over libzgl.
class CudaPathIntegrator : public Integrator {
public:
    explicit CudaPathIntegrator(int maxDepth) : mMaxDepth(maxDepth) {}
    ~CudaPathIntegrator() override {
        if (mZ) zgl_integrator_destroy(mZ);
    }

    bool init(zgl_scene* scene, int width, int height) override {
        zgl_integrator_params p;
        if (!ok(zgl_integrator_params_default(&p), "zgl_integrator_params_default")) return false;
        p.max_depth = mMaxDepth;
        mStatus.width = width;
        mStatus.height = height;
        return ok(zgl_integrator_create(scene, ZGL_INTEGRATOR_PATH, &p, &mZ), "zgl_integrator_create");
    }

    // NaivePath.cpp:77-105: a pending reset runs first, then one sample per pixel.
    bool renderOnePass() override {
        if (mShouldReset) {
            if (!reset(mStatus)) return false;
            mShouldReset = false;
        }
        return ok(zgl_integrator_render_pass(mZ, nullptr), "zgl_integrator_render_pass");
    }

    bool reset(const RenderStatus&) override { return ok(zgl_integrator_reset(mZ), "zgl_integrator_reset"); }

    float resultScale() const override {
        float s = 0.0f;
        zgl_integrator_result_scale(mZ, &s);
        return s;
    }

    bool readFrame(std::vector<float>& rgba, int32_t& spp) {
        rgba.assign((size_t)mStatus.width * mStatus.height * 4, 0.0f);
        return ok(zgl_integrator_frame(mZ, rgba.data(), &spp, nullptr), "zgl_integrator_frame");
    }

private:
    int mMaxDepth;
    zgl_integrator* mZ = nullptr;
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s scene.xml passes passes_after_reset max_depth out.bin\n", argv[0]);
        return 2;
    }
    const int passes = std::atoi(argv[2]), after = std::atoi(argv[3]), depth = std::atoi(argv[4]);
    zgl_scene* scene = nullptr;
    if (!ok(zgl_scene_load_xml(argv[1], 0, &scene), "zgl_scene_load_xml")) return 1;
    int32_t W = 0, H = 0;
    {
        int64_t info[13];
        if (!ok(zgl_scene_export(scene, "info", info, sizeof(info)), "zgl_scene_export")) return 1;
        W = (int32_t)info[0];
        H = (int32_t)info[1];
    }
    int rc = 0;
    {
        CudaPathIntegrator integ(depth);
        if (!integ.init(scene, W, H)) return 1;
        for (int i = 0; i < passes; i++)
            if (!integ.renderOnePass()) return 1;
        if (after > 0) {
            integ.setShouldReset();
            for (int i = 0; i < after; i++)
                if (!integ.renderOnePass()) return 1;
        }
        std::vector<float> frame;
        int32_t spp = 0;
        if (!integ.readFrame(frame, spp)) return 1;
        const float scale = integ.resultScale();
        FILE* f = std::fopen(argv[5], "wb");
        if (!f) return 1;
        std::fwrite(&W, 4, 1, f);
        std::fwrite(&H, 4, 1, f);
        std::fwrite(&spp, 4, 1, f);
        std::fwrite(&scale, 4, 1, f);
        if (std::fwrite(frame.data(), 4, frame.size(), f) != frame.size()) rc = 1;
        std::fclose(f);
    }
    zgl_scene_destroy(scene);
    return rc;
}
