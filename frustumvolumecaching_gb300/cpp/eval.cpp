/*
 * eval - the reference's evaluation program (src/eval.cu:88-497) on the C++
 * renderer API of fvc.hpp.
 *
 *   eval data camera-transforms output-dir [-sc] [-cp] [-w] [-wi] [-wc] [-or]
 *        [-r W H] [-nrit N]
 *
 * For every frame of the camera file: the plain render (timed over -nrit
 * iterations after one warm-up), a cache built at the frame's pose and the
 * cached render of it; then, around the focus point, 3 rotation offsets
 * (5, 10, 15 degrees) x 6 positions on a circle and 6 translations along the
 * view direction, each with a cache built at the offset pose and the cached
 * render of the original pose.  Writes <output-dir>/<image stem>/
 * {no_cache.png, cache.png, rot/<deg>/<theta>.png, trans/<step>.png,
 * metrics.json, timings.json} with the reference's file names and keys.
 *
 * -sc compares the plain render with the frame's PNG (when it can be read: the
 * dataset images are not part of this project) and the cached render with the
 * plain one (>= 35 dB, src/eval.cu:321), stopping at the first failure.
 * -wc (with -w) writes, for every rotation and translation offset, the
 * per-pixel compositing weight of the resampled and of the cached samples as
 * <name>_contr_new.png / <name>_contr_cache.png (gray, [0, 1] -> [0, 255];
 * src/eval.cu:381-410, 466-484).
 */
#include "fvc.hpp"

#include <array>
#include <iomanip>
#include <sstream>

namespace {

struct V3 {
    float x, y, z;
};
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 normalize(V3 a) { return (1.0f / std::sqrt(dot(a, a))) * a; }

/* rotation of v by `angle` about the unit axis k (Rodrigues' formula) */
V3 rotate(V3 v, float angle, V3 k)
{
    const float c = std::cos(angle), s = std::sin(angle);
    return c * v + s * cross(k, v) + ((1.0f - c) * dot(k, v)) * k;
}

/* camera-to-world matrix looking from eye at center: columns right, up, view, eye (src/eval.cu:74-84) */
CameraMatrix look_at(V3 eye, V3 center, V3 up)
{
    const V3 f = normalize(center - eye);
    const V3 r = normalize(cross(up, f));
    const V3 u = cross(f, r);
    return {make_float4(r.x, u.x, f.x, eye.x), make_float4(r.y, u.y, f.y, eye.y), make_float4(r.z, u.z, f.z, eye.z)};
}

struct Args {
    std::string data, transforms, out_dir;
    bool sanity = false, copy_orig = false, write_images = false, write_init = false, write_contrib = false, overwrite_res = false;
    int res_w = 1280, res_h = 720;
    unsigned n_iter = 1;
};

void usage()
{
    std::cout << "Usage: eval [-h] [--sanity-check] [--copy-original-images] [--write-images] [--write-cache-init-images]\n"
                 "            [--write-contrib-images] [--overwrite-resolution] [--resolution W H] [--num-render-iterations N]\n"
                 "            data camera-transforms output-dir\n";
}

/* the reference's argparse flags (src/eval.cu:90-108); a parse error prints the usage and exits 0 like it */
bool parse_args(int argc, char **argv, Args &a)
{
    std::vector<std::string> pos;
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        if (s == "-sc" || s == "--sanity-check") a.sanity = true;
        else if (s == "-cp" || s == "--copy-original-images") a.copy_orig = true;
        else if (s == "-w" || s == "--write-images") a.write_images = true;
        else if (s == "-wi" || s == "--write-cache-init-images") a.write_init = true;
        else if (s == "-wc" || s == "--write-contrib-images") a.write_contrib = true;
        else if (s == "-or" || s == "--overwrite-resolution") a.overwrite_res = true;
        else if (s == "-r" || s == "--resolution") {
            if (i + 2 >= argc) return false;
            a.res_w = std::atoi(argv[++i]);
            a.res_h = std::atoi(argv[++i]);
        } else if (s == "-nrit" || s == "--num-render-iterations") {
            if (i + 1 >= argc) return false;
            a.n_iter = (unsigned)std::strtoul(argv[++i], nullptr, 10);
        } else if (s == "-h" || s == "--help") {
            return false;
        } else if (!s.empty() && s[0] == '-') {
            return false;
        } else {
            pos.push_back(s);
        }
    }
    if (pos.size() != 3) return false;
    a.data = pos[0];
    a.transforms = pos[1];
    a.out_dir = pos[2];
    a.write_init = a.write_images && a.write_init;
    a.write_contrib = a.write_images && a.write_contrib;
    if (a.n_iter == 0) a.n_iter = 1;
    return true;
}

std::string json_str(const std::string &s)
{
    std::string o = "\"";
    for (char c : s) {
        if (c == '"' || c == '\\') o.push_back('\\');
        o.push_back(c);
    }
    return o + "\"";
}

std::string timings_json(const std::map<std::string, float> &t)
{
    std::ostringstream o;
    o << "{";
    bool first = true;
    for (const auto &kv : t) {
        o << (first ? "" : ",") << json_str(kv.first) << ":" << kv.second;
        first = false;
    }
    return o.str() + "}";
}

struct Perf {
    std::string image_name;
    int n_bricks_set, n_bricks_reserved;
    bool overflow;
    uint64_t n_cache_samples, n_resamples;
    std::string json() const
    {
        std::ostringstream o;
        o << "{\"image\":" << json_str(image_name) << ",\"n_bricks_set\":" << n_bricks_set << ",\"n_bricks_reserved\":" << n_bricks_reserved
          << ",\"overflow\":" << (overflow ? "true" : "false") << ",\"n_cache_samples\":" << n_cache_samples
          << ",\"n_resamples\":" << n_resamples << "}";
        return o.str();
    }
};

struct Timing {
    std::string image_name;
    float cache_init_ms, render_time_ms;
    std::map<std::string, float> timings;
    std::string json() const
    {
        std::ostringstream o;
        o << "{\"image\":" << json_str(image_name) << ",\"cache_init_ms\":" << cache_init_ms << ",\"render_time_ms\":" << render_time_ms
          << ",\"timings\":" << timings_json(timings) << "}";
        return o.str();
    }
};

template <typename T>
std::string json_list(const std::vector<T> &v)
{
    std::string o = "[";
    for (size_t i = 0; i < v.size(); ++i) o += (i ? "," : "") + v[i].json();
    return o + "]";
}

/* std::to_string(float) as the reference names translation images */
std::string float_name(float v) { return std::to_string(v); }

double now_ms() { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

/* RGBA8 PNG written by fvc_cpp::write_png (stored deflate blocks); false for any other encoding */
bool read_stored_png(const fs::path &p, int2 res, std::vector<uchar4> &out)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) return false;
    std::vector<uint8_t> d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (d.size() < 8 + 25 || d[1] != 'P') return false;
    size_t off = 8;
    std::vector<uint8_t> z;
    int w = 0, h = 0;
    while (off + 8 <= d.size()) {
        const uint32_t len = (uint32_t)d[off] << 24 | (uint32_t)d[off + 1] << 16 | (uint32_t)d[off + 2] << 8 | d[off + 3];
        const std::string type(d.begin() + off + 4, d.begin() + off + 8);
        if (off + 12 + len > d.size()) return false;
        const uint8_t *c = d.data() + off + 8;
        if (type == "IHDR") {
            w = (int)((uint32_t)c[0] << 24 | (uint32_t)c[1] << 16 | (uint32_t)c[2] << 8 | c[3]);
            h = (int)((uint32_t)c[4] << 24 | (uint32_t)c[5] << 16 | (uint32_t)c[6] << 8 | c[7]);
            if (c[8] != 8 || c[9] != 6 || c[12] != 0) return false;
        } else if (type == "IDAT") {
            z.insert(z.end(), c, c + len);
        }
        off += 12 + len;
    }
    if (w != res.x || h != res.y || z.size() < 2) return false;
    std::vector<uint8_t> raw;
    size_t q = 2;
    for (;;) {
        if (q + 5 > z.size() || (z[q] & 0x06) != 0) return false; /* only stored blocks */
        const bool last = z[q] & 1;
        const size_t len = z[q + 1] | (size_t)z[q + 2] << 8;
        q += 5;
        if (q + len > z.size()) return false;
        raw.insert(raw.end(), z.begin() + q, z.begin() + q + len);
        q += len;
        if (last) break;
    }
    if (raw.size() != (size_t)h * (1 + 4 * (size_t)w)) return false;
    out.resize((size_t)w * h);
    for (int y = 0; y < h; ++y) {
        if (raw[(size_t)y * (1 + 4 * w)] != 0) return false;
        std::memcpy(&out[(size_t)y * w], &raw[(size_t)y * (1 + 4 * w) + 1], 4 * (size_t)w);
    }
    return true;
}

}  // namespace

int main(int argc, char **argv)
{
    Args a;
    if (!parse_args(argc, argv, a)) {
        std::cout << "Argument parsing failed!" << std::endl;
        usage();
        return 0;
    }
    fs::create_directories(a.out_dir);

    LoaderData loader;
    if (!load_data(a.data, loader)) return 1;
    SceneInfo scene_info = loader.scene_info;
    StepsizeInfo stepsize = loader.stepsize_info;
    CameraInfo dataset_cam{};
    std::vector<CameraPathDataEntry> frames;
    if (!load_camerapath(a.transforms, loader.data_source, dataset_cam, frames)) return 1;

    RaymarchInfo dataset_rm{dataset_cam, {}, stepsize, 0, false, true};
    CameraInfo render_cam = dataset_cam, cache_cam = dataset_cam;
    if (a.overwrite_res) {
        render_cam.resize(make_int2(a.res_w, a.res_h));
        cache_cam.resize(make_int2(a.res_w, a.res_h));
    }
    RaymarchInfo cache_rm{cache_cam, {}, stepsize, 0, false, true};
    RaymarchInfo render_rm{render_cam, {}, stepsize, 0, false, true};

    ImageBuffer sanity_1(dataset_cam.resolution), sanity_2(dataset_cam.resolution);
    ImageBuffer render_image(render_cam.resolution), render_debug(render_cam.resolution);
    DebugData debug_data;
    DebugBuffer<float> contrib_resample(render_cam.resolution), contrib_cache(render_cam.resolution);
    debug_data.buffers = {&contrib_resample, &contrib_cache};

    CudaBuffer<uint8_t> &grid = loader.occupancy_grid_morton_bitfield;
    PerformanceRenderer renderer(scene_info, grid, loader.nerf_network);
    renderer.resizeRenderbuffers(render_cam.resolution);
    PerformanceRenderer sanity_renderer(scene_info, grid, loader.nerf_network);
    sanity_renderer.resizeRenderbuffers(dataset_cam.resolution);

    Cache cache;
    CacheSettings settings = CacheRenderer::default_cache_settings;
    settings.interpol_variant = loader.nerf_network.m_first_latent_is_density ? DensityIntermediates : Density;
    CachePerformanceRenderer cache_renderer(scene_info, grid, loader.nerf_network, &cache, &cache);
    cache_renderer.resizeCache(cache_cam.resolution, stepsize);
    cache_renderer.resizeRenderbuffers(cache_cam.resolution);
    cache_renderer.setCacheSettings(settings);

    const std::array<int, 3> view_degrees = {5, 10, 15};
    const int n_circle = 6;
    const float dt = stepsize.stepsize;
    const std::array<float, 6> translation_steps = {-0.25f, -0.1f, -dt * 0.5f, dt * 0.5f, 0.1f, 0.25f};
    const float PI = 3.14159265358979323846f;

    int i = 0;
    for (auto &entry : frames) {
        std::cerr << i << "/" << frames.size() << "\r" << std::flush;
        const std::string out_dir = a.out_dir + "/" + entry.image_path.stem().string();
        fs::create_directories(out_dir);
        const fs::path image_src = fs::path(a.transforms).remove_filename() / entry.image_path;
        if (a.copy_orig && fs::exists(image_src)) fs::copy(image_src, out_dir + "/orig.jpg", fs::copy_options::skip_existing);

        const CameraMatrix &cm = entry.transform_matrix;
        render_rm.cam_info.cam2world = cm;
        render_rm.cam_info.world2cam = cm.inverse();
        cache_rm.cam_info.cam2world = cm;
        cache_rm.cam_info.world2cam = cm.inverse();
        RaymarchInfo tmp_rm = dataset_rm;
        tmp_rm.cam_info.cam2world = cm;
        tmp_rm.cam_info.world2cam = cm.inverse();

        if (a.sanity) {
            std::vector<uchar4> ref;
            if (read_stored_png(image_src, dataset_cam.resolution, ref)) {
                sanity_1.upload(ref);
                sanity_renderer.render(tmp_rm, sanity_2);
                const float psnr = sanity_1.computePSNR(sanity_2, false, "");
                if (psnr < 15.f) {
                    std::cerr << "SANITY CHECK FAILED: " << entry.image_path.stem().string() << ", PSNR: " << psnr << std::endl;
                    sanity_2.writeToFile(out_dir + "/sanity_check_error.png");
                    break;
                }
            } else {
                std::cerr << "sanity check: " << image_src.string() << " not readable here, image check skipped" << std::endl;
            }
        }

        /* render without cache */
        renderer.render(render_rm, render_image);
        renderer._timer.reset();
        double t0 = now_ms();
        for (unsigned it = 0; it < a.n_iter; ++it) renderer.render(render_rm, render_image);
        const float render_time_new_ms = (float)(now_ms() - t0);
        std::vector<Perf> metrics_rot, metrics_trans;
        std::vector<Timing> timings_rot, timings_trans;
        const Timing no_cache{out_dir + "/no_cache", 0.0f, render_time_new_ms / a.n_iter, renderer._timer.getTimings(a.n_iter)};
        if (a.write_images) render_image.writeToFile(out_dir + "/no_cache.png");
        if (a.write_contrib) {
            contrib_resample.set(0.0f);
            contrib_cache.set(0.0f);
        }

        /* render with cache */
        cache_renderer.initCacheBlockwise(cache_rm, render_debug);
        cache_renderer.render(render_rm, render_image, a.write_contrib ? &debug_data : nullptr);
        if (a.sanity) {
            renderer.render(render_rm, render_image);
            cache_renderer.render(render_rm, render_debug);
            const float psnr = render_image.computePSNR(render_debug, false, "");
            if (psnr < 35.f) {
                std::cerr << "SANITY CHECK FAILED (CACHE RENDER): " << entry.image_path.stem().string() << ", PSNR: " << psnr << std::endl;
                render_debug.writeToFile(out_dir + "/sanity_check_error_cache.png");
                break;
            }
        }
        if (a.write_images) render_image.writeToFile(out_dir + "/cache.png");

        /* focus point: the camera position projected onto its view ray through the origin */
        const V3 view_dir = normalize({cm.m0.z, cm.m1.z, cm.m2.z});
        const V3 up = normalize({cm.m0.y, cm.m1.y, cm.m2.y});
        const V3 cam_pos = {cm.m0.w, cm.m1.w, cm.m2.w};
        const float proj = dot(-1.0f * cam_pos, view_dir);
        const V3 focus = cam_pos + proj * view_dir;
        const V3 cam_vec = cam_pos - focus;

        for (int deg : view_degrees) {
            const std::string sub = out_dir + "/rot/" + std::to_string(deg);
            if (a.write_images) fs::create_directories(sub);
            const float phi = float(deg) * PI / 180.f;
            const V3 start = rotate(cam_vec, phi, up);
            for (int ti = 0; ti < n_circle; ++ti) {
                const float theta = ti / (float)n_circle * (2.0f * PI);
                RaymarchInfo sub_rm = render_rm;
                const V3 pos = rotate(start, theta, normalize(cam_vec));
                sub_rm.cam_info.cam2world = look_at(focus + pos, focus, up);
                sub_rm.cam_info.world2cam = sub_rm.cam_info.cam2world.inverse();
                const std::string name = std::to_string(int(std::round(theta * 180.f / PI)));
                if (a.write_init) {
                    renderer.render(sub_rm, render_image);
                    render_image.writeToFile(sub + "/" + name + "_init.png");
                }
                t0 = now_ms();
                cache_renderer.initCacheBlockwise(sub_rm, render_debug);
                const float init_ms = (float)(now_ms() - t0);
                if (a.write_contrib) {
                    contrib_resample.set(0.0f);
                    contrib_cache.set(0.0f);
                }
                cache_renderer._timer.reset();
                t0 = now_ms();
                for (unsigned it = 0; it < a.n_iter; ++it)
                    cache_renderer.render(render_rm, render_image, a.write_contrib ? &debug_data : nullptr);
                const float rt = (float)(now_ms() - t0);
                if (a.write_images) render_image.writeToFile(sub + "/" + name + ".png");
                if (a.write_contrib) {
                    contrib_resample.writeToFile(sub + "/" + name + "_contr_new.png", createMinMaxConverter<float>(0.0f, 1.0f));
                    contrib_cache.writeToFile(sub + "/" + name + "_contr_cache.png", createMinMaxConverter<float>(0.0f, 1.0f));
                }
                const auto &is = cache_renderer._init_stats;
                const auto &rs = cache_renderer._render_stats;
                metrics_rot.push_back({std::to_string(deg) + "/" + name, is.n_bricks_set, is.n_bricks_reserved,
                                       is.n_bricks_set >= is.n_bricks_reserved, rs.n_cache_hits, rs.n_resamples});
                timings_rot.push_back({"r_" + std::to_string(deg) + "/" + name, init_ms, rt / a.n_iter, cache_renderer._timer.getTimings(a.n_iter)});
            }
        }

        const std::string sub = out_dir + "/trans";
        if (a.write_images) fs::create_directories(sub);
        for (float step : translation_steps) {
            RaymarchInfo sub_rm = render_rm;
            const V3 np = cam_pos + step * view_dir;
            sub_rm.cam_info.cam2world.m0.w = np.x;
            sub_rm.cam_info.cam2world.m1.w = np.y;
            sub_rm.cam_info.cam2world.m2.w = np.z;
            sub_rm.cam_info.world2cam = sub_rm.cam_info.cam2world.inverse();
            const std::string name = float_name(step);
            if (a.write_init) {
                renderer.render(sub_rm, render_image);
                render_image.writeToFile(sub + "/" + name + "_init.png");
            }
            t0 = now_ms();
            cache_renderer.initCacheBlockwise(sub_rm, render_debug);
            const float init_ms = (float)(now_ms() - t0);
            if (a.write_contrib) {
                contrib_resample.set(0.0f);
                contrib_cache.set(0.0f);
            }
            cache_renderer._timer.reset();
            t0 = now_ms();
            for (unsigned it = 0; it < a.n_iter; ++it)
                cache_renderer.render(render_rm, render_image, a.write_contrib ? &debug_data : nullptr);
            const float rt = (float)(now_ms() - t0);
            if (a.write_images) render_image.writeToFile(sub + "/" + name + ".png");
            if (a.write_contrib) {
                contrib_resample.writeToFile(sub + "/" + name + "_contr_new.png", createMinMaxConverter<float>(0.0f, 1.0f));
                contrib_cache.writeToFile(sub + "/" + name + "_contr_cache.png", createMinMaxConverter<float>(0.0f, 1.0f));
            }
            const auto &is = cache_renderer._init_stats;
            const auto &rs = cache_renderer._render_stats;
            metrics_trans.push_back({name, is.n_bricks_set, is.n_bricks_reserved, is.n_bricks_set >= is.n_bricks_reserved,
                                     rs.n_cache_hits, rs.n_resamples});
            timings_trans.push_back({"t_" + name, init_ms, rt / a.n_iter, cache_renderer._timer.getTimings(a.n_iter)});
        }

        std::ofstream(out_dir + "/metrics.json") << "{\"rot\":" << json_list(metrics_rot) << ",\"trans\":" << json_list(metrics_trans) << "}";
        std::ofstream(out_dir + "/timings.json") << "{\"no_cache\":" << no_cache.json() << ",\"rot\":" << json_list(timings_rot)
                                                 << ",\"trans\":" << json_list(timings_trans)
                                                 << ",\"render_time_new_ms\":" << render_time_new_ms / a.n_iter << "}";
        ++i;
    }
    return 0;
}
