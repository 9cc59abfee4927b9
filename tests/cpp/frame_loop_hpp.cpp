// A frame loop written against include/isti_renderer.hpp the way the
// reference's src/main.cu drives its Renderer: FrameData sized once, keyframe
// images read with ImageBuffer::readFromFile, FrameData::swap between keyframe
// pairs, every client frame rendered into one persistent RGBA8 buffer and
// written with ImageBuffer::writeToFile.
//
// usage: frame_loop_hpp <case dir> <out dir>
// <case dir>/case.txt (whitespace separated):
//   W H n_aux fill_r fill_g fill_b fill_a
//   n_aux lines: w h priority
//   n_pairs, then per pair:
//     per view (fwd, bwd, then curr and next of each aux camera):
//       has_motion has_shadows viewproj[16] inv_viewproj[16]   (column-major)
//     n_clients, then per client:
//       mode alpha frames_per_anchor shadow_frames_per_anchor no_shadows viewproj[16] inv_viewproj[16]
// Images: p<pair>_v<view>_{color.png, z.exr, motion.exr, shadowA.png,
// shadowB.png, shadowInfo.png}.  Output: <out dir>/NNNN.png, one per client
// frame in order; also <out dir>/average_z.txt = fwd z_buffer.average() of
// the last pair, and <out dir>/last_z.exr = that z_buffer written back.
#include "isti_renderer.hpp"

#include <cstdio>
#include <fstream>
#include <iostream>

namespace fs = std::filesystem;
using namespace isti;

static Mat4 read_mat(std::istream &in)
{
    float m[4][4];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            in >> m[c][r];
    return Mat4(m);
}

template <class T, int N>
static void read_optional(std::optional<ImageBuffer<T, N>> &opt, bool present, uint2 dims, const fs::path &file)
{
    if (!present)
    {
        opt = std::nullopt;
        return;
    }
    if (!opt.has_value())
    {
        opt.emplace();
        opt->resize(dims);
    }
    opt->readFromFile(file);
}

int main(int argc, char **argv)
{
    if (argc != 3)
    {
        std::fprintf(stderr, "usage: %s <case dir> <out dir>\n", argv[0]);
        return 2;
    }
    const fs::path case_dir = argv[1], out_dir = argv[2];
    try
    {
        std::ifstream in(case_dir / "case.txt");
        if (!in)
            throw std::runtime_error("cannot open case.txt");
        uint32_t W, H;
        int n_aux, fill[4];
        in >> W >> H >> n_aux >> fill[0] >> fill[1] >> fill[2] >> fill[3];
        std::vector<uint2> aux_res(n_aux);
        std::vector<int> aux_prio(n_aux);
        for (int i = 0; i < n_aux; i++)
            in >> aux_res[i].x >> aux_res[i].y >> aux_prio[i];

        FrameData frame_data{uint8_t(n_aux)};
        frame_data.resize(make_uint2(W, H), aux_res, aux_prio);

        Renderer renderer;
        renderer.setAutotune(true); // the frames must not depend on it
        ImageBuffer<uchar4, 4> render_buffer(make_uint2(W, H));
        render_buffer.memsetBuffer(make_uchar4(uint8_t(fill[0]), uint8_t(fill[1]), uint8_t(fill[2]), uint8_t(fill[3])));

        int n_pairs, frame_idx = 0;
        in >> n_pairs;
        for (int p = 0; p < n_pairs; p++)
        {
            if (p > 0)
                frame_data.swap();
            std::vector<MotionZBufferImage *> views{frame_data.fwd.get(), frame_data.bwd.get()};
            for (AuxCamData &a : frame_data.aux_cam_images)
            {
                views.push_back(a.curr.get());
                views.push_back(a.next.get());
            }
            for (size_t v = 0; v < views.size(); v++)
            {
                MotionZBufferImage &im = *views[v];
                int has_motion, has_shadows;
                in >> has_motion >> has_shadows;
                im.viewproj_mat = read_mat(in);
                im.inv_viewproj_mat = read_mat(in);
                const std::string stem = "p" + std::to_string(p) + "_v" + std::to_string(v) + "_";
                im.img.readFromFile(case_dir / (stem + "color.png"));
                im.z_buffer.readFromFile(case_dir / (stem + "z.exr"));
                read_optional(im.object_motion, has_motion != 0, im.dims, case_dir / (stem + "motion.exr"));
                read_optional(im.shadowColorA_img, has_shadows != 0, im.dims, case_dir / (stem + "shadowA.png"));
                read_optional(im.shadowColorB_img, has_shadows != 0, im.dims, case_dir / (stem + "shadowB.png"));
                read_optional(im.shadowInfo_img, has_shadows != 0, im.dims, case_dir / (stem + "shadowInfo.png"));
            }
            int n_clients;
            in >> n_clients;
            for (int c = 0; c < n_clients; c++)
            {
                int mode, fpa, sfpa, no_shadows;
                float alpha;
                in >> mode >> alpha >> fpa >> sfpa >> no_shadows;
                RenderInfo info{make_uint2(W, H), alpha, read_mat(in), read_mat(in),
                                AdditionalRenderInfo{fpa, sfpa, no_shadows != 0, RenderMode(mode)}};
                if (!in)
                    throw std::runtime_error("case.txt is truncated");
                renderer.render(render_buffer, info, frame_data);
                if (renderer.last_status() != ISTI_OK) // printed by render, like the reference
                    return 1;
                char name[32];
                std::snprintf(name, sizeof name, "%04d.png", frame_idx++);
                render_buffer.writeToFile(out_dir / name);
            }
        }
        std::ofstream(out_dir / "average_z.txt") << std::hexfloat << frame_data.fwd->z_buffer.average() << "\n";
        frame_data.fwd->z_buffer.writeToFile(out_dir / "last_z.exr");
        std::printf("frames %d\n", frame_idx);
    }
    catch (const Error &e)
    {
        std::fprintf(stderr, "isti error %d: %s\n", int(e.status), e.what());
        return 1;
    }
    catch (const std::exception &e)
    {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
