// Error behaviour of include/isti_renderer.hpp, as in the reference: a failing render
// is printed and execution continues (Renderer::last_status() has the status); a
// resize to another size and an unreadable file throw std::runtime_error.  Runs
// with or without a GPU (without one, the renderer is not created and says so).
#include "isti_renderer.hpp"

#include <cstdio>

using namespace isti;

int main()
{
    Renderer renderer;
    FrameData frame_data{0}; // views never sized: the render is rejected
    ImageBuffer<uchar4, 4> out(make_uint2(8u, 8u));
    const RenderInfo info{make_uint2(8u, 8u), 0.5f, Mat4(), Mat4(), AdditionalRenderInfo{4, 4, false, OURS}};
    renderer.render(out, info, frame_data);
    std::printf("render status %d\n", int(renderer.last_status()));
    try
    {
        out.resize(make_uint2(4u, 4u));
        std::printf("resize did not throw\n");
    }
    catch (const std::runtime_error &e)
    {
        std::printf("resize threw: %s\n", e.what());
    }
    try
    {
        out.readFromFile("does_not_exist.png");
        std::printf("read did not throw\n");
    }
    catch (const std::runtime_error &e)
    {
        std::printf("read threw: %s\n", e.what());
    }
    try
    {
        ImageBuffer<float, 1> z(make_uint2(8u, 8u));
        z.readFromFile("does_not_exist.exr");
        std::printf("exr read did not throw\n");
    }
    catch (const std::runtime_error &e)
    {
        std::printf("exr read threw: %s\n", e.what());
    }
    return 0;
}
