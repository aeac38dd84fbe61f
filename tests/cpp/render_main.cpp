// Headless replacement of the reference's main loop (Core/Core.cpp:20-31,
// 239-438) written against include/venu_core.hpp.  The lines marked with a
// Core/Core.cpp line number are the reference's own statements, unchanged;
// the GLFW / OpenGL / ImGui display between them is replaced by reading the
// pixels back and writing a binary PPM, the raw RGBA8 bytes and a PFM.  The
// image size comes from the command line (the reference fixes 1200 wide at
// 3:2).  Used by tests/test_cpp_dropin.py.
//
//   render_main <width> <height> <frames> <out.ppm> <out.rgba> [out.pfm] [zero_copy]
//   render_main gl        (constructs a GL_INTEROP buffer: must throw, exit 0 if it does)
#include <cstdio>
#include <cstdlib>
#include <string>

#include "venu_core.hpp"

using namespace venu_core;

int main(int argc, char** argv) {
    if (argc == 2 && std::string(argv[1]) == "gl") {
        try {
            CUDAOutputBuffer<uchar4> gl(CUDAOutputBufferType::GL_INTEROP, 4, 4);
        } catch (const Exception& e) {
            return e.status == VENU_ERR_INVALID ? 0 : 4;
        }
        return 5;
    }
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s W H frames out.ppm out.rgba [out.pfm]\n", argv[0]);
        return 2;
    }
    const int image_width = std::atoi(argv[1]);
    const int image_height = std::atoi(argv[2]);
    const int frames = std::atoi(argv[3]);
    try {
        // Core/Core.cpp:21-26 with the aspect ratio of the requested size
        vec3 lookfrom{13, 2, 3};
        vec3 lookat{0, 0, 0};
        auto dist_to_focus = 10.0f;
        auto aperture = 0.1f;
        const auto aspect_ratio = (float)image_width / (float)image_height;
        Camera camera(lookfrom, 20.0f, aspect_ratio, aperture, dist_to_focus);  // Core/Core.cpp:29
        Scene scene;                                                             // Core/Core.cpp:30
        Renderer optix_renderer;                                                 // Core/Core.cpp:31
        std::string ptxSource;  // no PTX: the kernels are in libvenusaur_gb300
        optix_renderer.Init(scene, ptxSource);  // Core/Core.cpp:246
        const bool zero_copy = argc > 7 && std::string(argv[7]) == "zero_copy";
        if (zero_copy) {  // the ZERO_COPY type: the pixels in mapped host memory
            CUDAOutputBuffer<uchar4> zc(CUDAOutputBufferType::ZERO_COPY, image_width, image_height);
            camera.SetForward(lookat - lookfrom);
            for (int f = 0; f < frames; ++f) optix_renderer.Draw(camera, zc);
            const uchar4* px = zc.getHostPointer();
            FILE* g = std::fopen(argv[5], "wb");
            if (!g) return 3;
            std::fwrite(px, sizeof(uchar4), (size_t)image_width * image_height, g);
            std::fclose(g);
            optix_renderer.Cleanup();
            return 0;
        }
        CUDAOutputBuffer<uchar4> outputBuffer(CUDAOutputBufferType::CUDA_DEVICE, image_width, image_height);  // Core/Core.cpp:252
        camera.SetForward(lookat - lookfrom);  // Core/Core.cpp:353
        for (int f = 0; f < frames; ++f) {
            optix_renderer.Draw(camera, outputBuffer);  // Core/Core.cpp:394
        }
        const uchar4* px = outputBuffer.getHostPointer();
        FILE* g = std::fopen(argv[5], "wb");
        if (!g) return 3;
        std::fwrite(px, sizeof(uchar4), (size_t)image_width * image_height, g);
        std::fclose(g);
        outputBuffer.writePPM(argv[4]);
        if (argc > 6) outputBuffer.writePFM(argv[6]);
        optix_renderer.Cleanup();  // Core/Core.cpp:432
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
