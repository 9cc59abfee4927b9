// C entry point around the reference's own Renderer (src/renderer.cu, compiled
// on the host through isti_refhost.h).  Test infrastructure only: it turns
// plain host arrays into the reference's FrameData / RenderInfo
// (include/data.h:79-116, include/renderer.h:18-35), runs Renderer::render
// (src/renderer.cu:607-694) and copies out the output image, the 64-bit
// splat buffers and the flow fields.
//
// View order for the per-view outputs: fwd main, bwd main, then for each aux
// camera i: curr (forward keyframe), next (backward keyframe).

// The splat buffers and flow fields are private members of Renderer
// (include/renderer.h:58-92); this harness reads them back for the bit-exact
// splat-key checks.
#define private public
#include "renderer_host.cpp" // generated from src/renderer.cu by build_ref.py
#undef private

#include "../isti_oracle.h"

namespace isti_refhost
{
void reset_all();
}

namespace
{
glm::mat4 to_mat(const float *m)
{
    glm::mat4 r;
    for (int c = 0; c < 4; c++)
        for (int rr = 0; rr < 4; rr++)
            r[c][rr] = m[c * 4 + rr];
    return r;
}

void fill(MotionZBufferImage &img, const oracle_view &v)
{
    img.img.upload(reinterpret_cast<uchar4 *>(const_cast<uint8_t *>(v.color)));
    img.z_buffer.upload(const_cast<float *>(v.z));
    if (v.motion)
        img.object_motion.value().upload(reinterpret_cast<float4 *>(const_cast<float *>(v.motion)));
    else
        img.object_motion = std::nullopt;
    auto opt_upload = [](std::optional<ImageBuffer<uchar4, 4>> &buf, const uint8_t *src) {
        if (src)
            buf.value().upload(reinterpret_cast<uchar4 *>(const_cast<uint8_t *>(src)));
        else
            buf = std::nullopt;
    };
    opt_upload(img.shadowColorA_img, v.shadow_color_a);
    opt_upload(img.shadowColorB_img, v.shadow_color_b);
    opt_upload(img.shadowInfo_img, v.shadow_info);
    img.viewproj_mat = to_mat(v.viewproj);
    img.inv_viewproj_mat = to_mat(v.inv_viewproj);
}

void export_view(oracle_view_out &o, uint64_cu *splat, ImageBuffer<float4, 4> &cam_ff, ImageBuffer<float4, 4> &full_ff, uint2 dims)
{
    const size_t n = (size_t)dims.x * dims.y;
    if (o.splat)
        std::memcpy(o.splat, splat, n * sizeof(uint64_t));
    if (o.cam_ff)
        cam_ff.download(reinterpret_cast<float4 *>(o.cam_ff));
    if (o.full_ff)
        full_ff.download(reinterpret_cast<float4 *>(o.full_ff));
}
} // namespace

extern "C" int isti_ref_render(const oracle_frame *frame, const oracle_render_info *info, uint8_t *out_rgba, oracle_view_out *outs)
{
    int rc = 0;
    try
    {
        const int n_aux = frame->num_aux;
        // Renderer::_curr_resolution has no initialiser (include/renderer.h:86) and
        // resizeBuffers only allocates the splat buffers when it differs from the
        // render resolution (src/renderer.cu:575).  Construct in zeroed storage so a
        // Renderer placed in recycled heap memory still allocates them.
        void *storage = std::calloc(1, sizeof(Renderer));
        if (!storage)
            throw std::bad_alloc();
        struct Destroy
        {
            void operator()(Renderer *p) const
            {
                p->~Renderer();
                std::free(p);
            }
        };
        std::unique_ptr<Renderer, Destroy> renderer(new (storage) Renderer());
        std::unique_ptr<FrameData> fd(new FrameData((uint8_t)n_aux));
        std::vector<uint2> aux_res;
        std::vector<int> aux_prio;
        for (int i = 0; i < n_aux; i++)
        {
            aux_res.push_back(make_uint2(frame->aux_curr[i].width, frame->aux_curr[i].height));
            aux_prio.push_back(frame->aux_priority ? frame->aux_priority[i] : 0);
        }
        fd->resize(make_uint2(frame->fwd.width, frame->fwd.height), aux_res, aux_prio);
        fill(*fd->fwd, frame->fwd);
        fill(*fd->bwd, frame->bwd);
        for (int i = 0; i < n_aux; i++)
        {
            fill(*fd->aux_cam_images[i].curr, frame->aux_curr[i]);
            fill(*fd->aux_cam_images[i].next, frame->aux_next[i]);
        }

        RenderInfo ri{make_uint2(info->width, info->height), info->alpha, to_mat(info->viewproj), to_mat(info->inv_viewproj),
                      {info->frames_per_anchor, info->shadow_frames_per_anchor, info->no_shadows != 0, (RenderMode)info->mode}};

        ImageBuffer<uchar4, 4> out(make_uint2(info->width, info->height));
        out.upload(reinterpret_cast<uchar4 *>(out_rgba));
        renderer->render(out, ri, *fd);
        out.download(reinterpret_cast<uchar4 *>(out_rgba));

        if (outs && info->mode != TIMEWARP)
        {
            export_view(outs[0], renderer->d_fwd_main_splatting_buffer, renderer->fwd2cam_ff, renderer->fwd2bwd_ff, fd->fwd->dims);
            export_view(outs[1], renderer->d_bwd_main_splatting_buffer, renderer->bwd2cam_ff, renderer->bwd2fwd_ff, fd->bwd->dims);
            for (int i = 0; i < n_aux; i++)
            {
                export_view(outs[2 + 2 * i], renderer->d_aux_cam_splatting_buffers[i].forward, renderer->fwd2cam_aux_ff[i],
                            renderer->fwd2bwd_aux_ff[i], fd->aux_cam_images[i].curr->dims);
                export_view(outs[3 + 2 * i], renderer->d_aux_cam_splatting_buffers[i].backward, renderer->bwd2cam_aux_ff[i],
                            renderer->bwd2fwd_aux_ff[i], fd->aux_cam_images[i].next->dims);
            }
        }
    }
    catch (const std::exception &ex)
    {
        std::fprintf(stderr, "isti_ref_render: %s\n", ex.what());
        rc = -1;
    }
    isti_refhost::reset_all();
    return rc;
}
