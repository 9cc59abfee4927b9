// splinter — the reference's command-line frame loop (src/main.cu), over the
// C ABI of libisti: keyframes from a dataset folder (include/isti_dataset.h),
// client frames rendered by isti_render (include/isti.h), optionally written
// as PNG files.
//
//   splinter <input-dir> <output-dir> [-c cam-dir] [-w] [-r W H] [-a dir...]
//            [-l n] [-m 0..4] [-lh] [-ns] [-hb] [--timing]
//
// Same flags, defaults and loop as src/main.cu:66-191: client frames at the
// camera path's clientFps (120 Hz for 15 s without -c), frames_per_anchor =
// clientFps / serverFps, keyframe reads at b == latency (or at the end of the
// interval when the latency reaches it), t = (fpa + b) / fpa for frames
// rendered before the new keyframe arrives, hold-last skips those frames,
// holes-black clears the output before each frame.  --timing (not in the
// reference) prints one JSON line with load and render times.
#include "isti.h"
#include "isti_dataset.h"
#include "isti_io.h"
#include "isti_mat4.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <filesystem>
#include <iomanip>
#include <iostream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace fs = std::filesystem;
using isti::host::mat4;

namespace
{
struct Args
{
    std::string input, output, camera_path;
    bool write_images = false, hold_last = false, no_shadows = false, holes_black = false, timing = false;
    int width = 2560, height = 1440; // the reference's default resolution
    std::vector<std::string> aux;
    int latency = 0, mode = 0;
};

const char *USAGE =
    "Usage: splinter [-h] [--camera-path VAR] [--write-images] [--resolution VAR VAR] [--aux-dirs VAR...]\n"
    "                [--latency VAR] [--mode VAR] [--latency-hold-last] [--no-shadows] [--holes-black]\n"
    "                [--timing] input-dir output-dir\n"
    "\n"
    "Splinter - Split-Rendering Frame Interpolation\n"
    "\n"
    "Positional arguments:\n"
    "  input-dir                  path to the input directory\n"
    "  output-dir                 path to the output directory\n"
    "\n"
    "Optional arguments:\n"
    "  -h, --help                 shows help message and exits\n"
    "  -c, --camera-path          input camera path\n"
    "  -w, --write-images         write images to output directory\n"
    "  -r, --resolution           rendering resolution [nargs: 2] [default: {2560 1440}]\n"
    "  -a, --aux-dirs             auxilliary cam directory names [nargs: 1 or more]\n"
    "  -l, --latency              delay of server frames by <l> client frames [default: 0]\n"
    "  -m, --mode                 rendering mode (for benchmarking; see RenderMode) [default: 0]\n"
    "  -lh, --latency-hold-last   hold the last frame when latency sets in\n"
    "  -ns, --no-shadows          manually disables dynamic shadows, even when information is present\n"
    "  -hb, --holes-black         manually disable hole filling; holes will be left black\n"
    "      --timing               print one JSON line with load and render times\n";

bool parse_int(const std::string &s, int &out)
{
    char *end = nullptr;
    errno = 0;
    const long v = std::strtol(s.c_str(), &end, 10);
    if (errno || !end || *end || s.empty() || v < INT32_MIN || v > INT32_MAX)
        return false;
    out = int(v);
    return true;
}

// Returns an empty string on success, else the parse error.
std::string parse_args(int argc, char **argv, Args &a, bool &help)
{
    std::vector<std::string> pos;
    auto is_option = [](const std::string &s) { return s.size() > 1 && s[0] == '-' && !(s[1] >= '0' && s[1] <= '9'); };
    for (int i = 1; i < argc; i++)
    {
        const std::string s = argv[i];
        auto value = [&](std::string &out) -> bool {
            if (i + 1 >= argc)
                return false;
            out = argv[++i];
            return true;
        };
        auto int_value = [&](int &out) -> bool {
            std::string v;
            return value(v) && parse_int(v, out);
        };
        if (s == "-h" || s == "--help")
            help = true;
        else if (s == "-c" || s == "--camera-path")
        {
            if (!value(a.camera_path))
                return s + ": expected 1 argument";
        }
        else if (s == "-w" || s == "--write-images")
            a.write_images = true;
        else if (s == "-r" || s == "--resolution")
        {
            if (!int_value(a.width) || !int_value(a.height))
                return s + ": expected 2 integer arguments";
        }
        else if (s == "-a" || s == "--aux-dirs")
        {
            a.aux.clear();
            while (i + 1 < argc && !is_option(argv[i + 1]))
                a.aux.push_back(argv[++i]);
            if (a.aux.empty())
                return s + ": expected at least 1 argument";
        }
        else if (s == "-l" || s == "--latency")
        {
            if (!int_value(a.latency))
                return s + ": expected an integer";
        }
        else if (s == "-m" || s == "--mode")
        {
            if (!int_value(a.mode) || a.mode < 0 || a.mode > 4)
                return s + ": invalid choice (expected 0, 1, 2, 3 or 4)";
        }
        else if (s == "-lh" || s == "--latency-hold-last")
            a.hold_last = true;
        else if (s == "-ns" || s == "--no-shadows")
            a.no_shadows = true;
        else if (s == "-hb" || s == "--holes-black")
            a.holes_black = true;
        else if (s == "--timing")
            a.timing = true;
        else if (is_option(s))
            return "Unknown argument: " + s;
        else
            pos.push_back(s);
    }
    if (help)
        return "";
    if (pos.size() < 2)
        return pos.empty() ? "input-dir: 1 argument(s) expected. 0 provided." : "output-dir: 1 argument(s) expected. 0 provided.";
    if (pos.size() > 2)
        return "Maximum number of positional arguments exceeded";
    a.input = pos[0];
    a.output = pos[1];
    return "";
}

mat4 mat_of(const float *v)
{
    mat4 m;
    std::memcpy(m.m, v, sizeof(m.m));
    return m;
}

// Encodes and writes the PNG files on worker threads, so that encoding overlaps the
// rendering of the next frames (the reference encodes on the render thread).  At most
// `max_queued` frames wait; submit() blocks beyond that.
class PngWriterPool
{
public:
    PngWriterPool(unsigned n_threads, size_t max_queued) : max_queued_(max_queued)
    {
        for (unsigned i = 0; i < n_threads; i++)
            threads_.emplace_back([this] { work(); });
    }
    ~PngWriterPool()
    {
        std::string ignored;
        finish(ignored);
    }
    void submit(std::string path, std::vector<uint8_t> rgba, int32_t w, int32_t h)
    {
        std::unique_lock<std::mutex> lock(m_);
        room_.wait(lock, [&] { return queue_.size() < max_queued_; });
        queue_.push_back(Job{std::move(path), std::move(rgba), w, h});
        ready_.notify_one();
    }
    // waits for every submitted frame; false (with the first error) if one failed
    bool finish(std::string &err)
    {
        {
            std::lock_guard<std::mutex> lock(m_);
            stop_ = true;
        }
        ready_.notify_all();
        for (std::thread &t : threads_)
            if (t.joinable())
                t.join();
        err = error_;
        return error_.empty();
    }

private:
    struct Job
    {
        std::string path;
        std::vector<uint8_t> rgba;
        int32_t w, h;
    };
    void work()
    {
        for (;;)
        {
            Job job;
            {
                std::unique_lock<std::mutex> lock(m_);
                ready_.wait(lock, [&] { return stop_ || !queue_.empty(); });
                if (queue_.empty())
                    return;
                job = std::move(queue_.front());
                queue_.pop_front();
                room_.notify_one();
            }
            if (isti_png_encode_file(job.path.c_str(), job.w, job.h, 4, job.rgba.data()) != ISTI_OK)
            {
                std::lock_guard<std::mutex> lock(m_);
                if (error_.empty())
                    error_ = isti_last_error();
            }
        }
    }
    size_t max_queued_;
    std::vector<std::thread> threads_;
    std::deque<Job> queue_;
    std::mutex m_;
    std::condition_variable ready_, room_;
    bool stop_ = false;
    std::string error_;
};

int fail(const std::string &what)
{
    std::cout << std::endl << "Error - " << what << std::endl;
    return 1;
}

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
} // namespace

int main(int argc, char **argv)
{
    Args args;
    bool help = false;
    const std::string perr = parse_args(argc, argv, args, help);
    if (help)
    {
        std::cout << USAGE;
        return 0;
    }
    if (!perr.empty())
    {
        std::cout << "Error - Argument parsing failed!" << std::endl << perr << std::endl << USAGE;
        return 1;
    }
    if (!fs::exists(args.input))
    {
        std::cout << "Input directory invalid" << std::endl;
        return 1;
    }
    std::error_code ec;
    if (!fs::exists(args.output) && !fs::create_directories(args.output, ec))
    {
        std::cout << "Output directory could not be created" << std::endl;
        return 1;
    }

    cudaStream_t stream = nullptr;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail("no CUDA device");

    double load_s = 0.0, render_s = 0.0, write_s = 0.0;
    auto t_load = std::chrono::steady_clock::now();
    std::vector<const char *> aux_dirs;
    for (const std::string &s : args.aux)
        aux_dirs.push_back(s.c_str());
    isti_dataset *data = nullptr;
    if (isti_dataset_open(args.input.c_str(), int32_t(aux_dirs.size()), aux_dirs.data(), stream, &data) != ISTI_OK)
        return fail(isti_last_error());
    load_s += seconds_since(t_load);

    isti_camera_info main_cam{};
    isti_dataset_camera(data, -1, &main_cam);
    isti_camera_path *cam_path = nullptr;
    isti_camera_info path_info{};
    const bool use_input_cam = !args.camera_path.empty();
    if (use_input_cam)
    {
        if (isti_camera_path_open(args.camera_path.c_str(), &cam_path) != ISTI_OK)
            return fail(isti_last_error());
        isti_camera_path_info(cam_path, &path_info);
    }

    const uint32_t w = uint32_t(args.width), h = uint32_t(args.height);
    if (args.width <= 0 || args.height <= 0)
        return fail("resolution must be positive");
    void *d_out = nullptr;
    const size_t out_bytes = size_t(w) * h * 4;
    if (cudaMalloc(&d_out, out_bytes) != cudaSuccess || cudaMemsetAsync(d_out, 0, out_bytes, stream) != cudaSuccess)
        return fail("cannot allocate the output image");
    const unsigned n_writers = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    PngWriterPool writers(args.write_images ? n_writers : 0, 2 * n_writers);
    isti_renderer *renderer = nullptr;
    if (isti_renderer_create(&renderer) != ISTI_OK)
        return fail(isti_last_error());

    const int fixed_client_fps = 120, fixed_duration_s = 15;
    const int total_n_frames = use_input_cam ? path_info.n_frames : fixed_client_fps * fixed_duration_s;
    const int client_fps = use_input_cam ? path_info.client_fps : fixed_client_fps;
    if (main_cam.server_fps <= 0 || client_fps / main_cam.server_fps <= 0)
        return fail("clientFps / serverFps must be at least 1");
    const int fpa = client_fps / main_cam.server_fps;
    const int sfpa = main_cam.shadow_fps / main_cam.server_fps;
    const int latency = args.latency;
    int rendered = 0;

    auto read_next = [&]() -> bool {
        const auto t0 = std::chrono::steady_clock::now();
        int32_t advanced = 0;
        const bool ok = isti_dataset_read_next(data, &advanced) == ISTI_OK;
        load_s += seconds_since(t0);
        return ok;
    };

    for (int i = 0; i < total_n_frames; i += fpa)
    {
        for (int b = 0; b < fpa; b++)
        {
            if (latency == b && !read_next())
                return fail(isti_last_error());
            const int frame_number = i + b + 1;
            if (frame_number > total_n_frames)
                break;
            const float t = float(latency > b ? fpa + b : b) / float(fpa);
            mat4 view, proj;
            if (use_input_cam)
            {
                isti_camera_frame cf{};
                isti_camera_path_frame(cam_path, i + b, &cf);
                view = mat_of(cf.w2c);
                float p[16];
                isti_normalize_proj(cf.proj, p);
                proj = mat_of(p);
            }
            else
            {
                float v0[16], v1[16], p0[16];
                isti_dataset_matrices(data, 0, v0, p0);
                isti_dataset_matrices(data, 1, v1, nullptr);
                view = isti::host::interpolate(mat_of(v0), mat_of(v1), t); // getIntermediateViewMatrix (main.cu:26-28)
                proj = mat_of(p0);
            }
            const mat4 vp = isti::host::mul(proj, view);
            const mat4 ivp = isti::host::inverse(vp);

            std::cout << "Frame: " << std::setfill(' ') << std::setw(3) << frame_number << " / " << std::setfill(' ')
                      << std::setw(3) << total_n_frames << "\r";
            std::flush(std::cout);

            const auto t0 = std::chrono::steady_clock::now();
            if (args.holes_black && cudaMemsetAsync(d_out, 0, out_bytes, stream) != cudaSuccess)
                return fail("cudaMemsetAsync failed");
            if (!(b < latency && args.hold_last)) // hold the last frame while the keyframe is late
            {
                isti_render_info info{};
                info.width = w;
                info.height = h;
                info.alpha = t;
                std::memcpy(info.viewproj, vp.m, sizeof(info.viewproj));
                std::memcpy(info.inv_viewproj, ivp.m, sizeof(info.inv_viewproj));
                info.frames_per_anchor = fpa;
                info.shadow_frames_per_anchor = sfpa;
                info.no_shadows = args.no_shadows;
                info.mode = args.mode;
                isti_frame_data fd{};
                isti_dataset_frame(data, &fd);
                if (isti_render(renderer, d_out, &info, &fd, stream) != ISTI_OK)
                    return fail(isti_last_error());
                rendered++;
            }
            if (args.write_images)
            {
                std::vector<uint8_t> host_img(out_bytes);
                if (cudaMemcpyAsync(host_img.data(), d_out, out_bytes, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                    cudaStreamSynchronize(stream) != cudaSuccess)
                    return fail("cannot read the output image");
                render_s += seconds_since(t0);
                const auto t1 = std::chrono::steady_clock::now();
                std::ostringstream name;
                name << std::setfill('0') << std::setw(4) << (frame_number - 1) << ".png";
                writers.submit((fs::path(args.output) / name.str()).string(), std::move(host_img), int32_t(w), int32_t(h));
                write_s += seconds_since(t1);
            }
            else
            {
                if (cudaStreamSynchronize(stream) != cudaSuccess)
                    return fail("render failed");
                render_s += seconds_since(t0);
            }
            if (latency > b && b == fpa - 1 && !read_next()) // the keyframe arrives after the whole interval
                return fail(isti_last_error());
        }
    }
    std::cout << std::endl;
    {
        const auto t1 = std::chrono::steady_clock::now();
        std::string werr;
        if (!writers.finish(werr))
            return fail(werr);
        write_s += seconds_since(t1);
    }

    int32_t dev_status = 0;
    isti_renderer_device_status(renderer, &dev_status);
    if (args.timing)
        std::cout << "{\"frames\": " << total_n_frames << ", \"rendered\": " << rendered << ", \"load_s\": " << load_s
                  << ", \"render_s\": " << render_s << ", \"write_s\": " << write_s << ", \"device_status\": " << dev_status
                  << "}" << std::endl;
    isti_renderer_destroy(renderer);
    isti_camera_path_close(cam_path);
    isti_dataset_close(data);
    cudaFree(d_out);
    cudaStreamDestroy(stream);
    if (dev_status != 0)
    {
        std::cout << "Error - a kernel reported status " << dev_status << " (" << isti_status_string(isti_status(dev_status))
                  << ")" << std::endl;
        return 2;
    }
    return 0;
}
