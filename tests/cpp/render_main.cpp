// Headless replacement of the reference's main loop (Core/Core.cpp:239-438)
// written against include/venu_core.hpp: Init, two Draws, read back, write a
// binary PPM, the raw RGBA8 bytes and optionally a PFM.  Used by tests/test_cpp_dropin.py.
//
//   render_main <width> <height> <spp> <max_depth> <out.ppm> <out.rgba> [out.pfm]
#include <cstdio>
#include <cstdlib>

#include "venu_core.hpp"

using namespace venu_core;

int main(int argc, char** argv) {
    if (argc < 7) {
        std::fprintf(stderr, "usage: %s W H spp depth out.ppm out.rgba\n", argv[0]);
        return 2;
    }
    const int W = std::atoi(argv[1]), H = std::atoi(argv[2]);
    const uint32_t spp = (uint32_t)std::atoi(argv[3]), depth = (uint32_t)std::atoi(argv[4]);
    try {
        // Core/Core.cpp:21-30 with aspect = W/H
        vec3 lookfrom(13, 2, 3), lookat(0, 0, 0);
        Camera camera(lookfrom, 20.0f, (float)W / (float)H, 0.1f, 10.0f);
        Scene scene;
        Renderer renderer(spp, depth);
        renderer.Init(scene);
        CUDAOutputBuffer out(W, H);
        camera.SetForward(vec3(lookat.x - lookfrom.x, lookat.y - lookfrom.y, lookat.z - lookfrom.z));
        renderer.Draw(camera, out);
        renderer.Draw(camera, out);
        std::vector<uint8_t> px = out.getHostPointer();
        out.writePPM(argv[5]);
        if (argc > 7) out.writePFM(argv[7]);
        renderer.Cleanup();
        FILE* g = std::fopen(argv[6], "wb");
        if (!g) return 3;
        std::fwrite(px.data(), 1, px.size(), g);
        std::fclose(g);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
