/*
 * render_path - the real-time viewer's camera-path rendering
 * (Application::renderCameraPath, realtime_viewer/src/application.cu:248-336)
 * without a window: frames are written as PNG files.
 *
 *   render_path data camera_path.json output-dir [-frames N] [-spp N] [-r W H]
 *               [-cache] [-auto] [-cache-r W H] [-eval T0 T1 N]
 *
 * For path frame i of n = duration * fps: the camera at play time i / n from
 * the key-frame spline, the next frame's pose as the motion-blur end pose
 * (motion blur on, deterministic off, as the viewer renders paths), focal
 * length from the path's horizontal field of view.  With render_from_cache
 * (-cache, or the file's settings) the cache is rebuilt at the pose half a
 * frame ahead whenever the cache-update rule asks (every frame unless
 * auto_cache_update; with it, when the last frame's hit ratio fell below
 * cache_min_hit_ratio or the camera moved farther than
 * cache_update_distance from the last build), at the cache resolution and
 * with the sampling rate doubled, as the viewer's initCache does
 * (application.cu:132-158).  Each frame accumulates spp samples
 * (sample_index 0..spp-1) in the progressive image, is written to
 * <output-dir>/frame_<i, 6 digits>.png and logged to <output-dir>/frames.json
 * (cache update, hit ratio, samples per pixel, milliseconds).  The viewer
 * then calls ffmpeg on the frames; this program stops at the frames.
 *
 * -eval T0 T1 N prints N cameras of the spline at t = T0..T1 as JSON lines
 * (cam2world rows, aperture, focus) and renders nothing.
 */
#include "fvc_camera_path.hpp"

#include <cstdio>
#include <iomanip>

namespace {

struct Args {
    std::string data, path, out_dir;
    int frames = -1, spp = -1, res_w = 0, res_h = 0, cache_w = 0, cache_h = 0;
    bool cache = false, auto_update = false;
    bool eval = false;
    float t0 = 0.f, t1 = 1.f;
    int n_eval = 0;
};

bool parse(int argc, char **argv, Args &a)
{
    int pos = 0;
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        auto need = [&](int n) { return i + n < argc; };
        if (s == "-frames" && need(1)) a.frames = std::atoi(argv[++i]);
        else if (s == "-spp" && need(1)) a.spp = std::atoi(argv[++i]);
        else if (s == "-r" && need(2)) { a.res_w = std::atoi(argv[++i]); a.res_h = std::atoi(argv[++i]); }
        else if (s == "-cache-r" && need(2)) { a.cache_w = std::atoi(argv[++i]); a.cache_h = std::atoi(argv[++i]); }
        else if (s == "-cache") a.cache = true;
        else if (s == "-auto") a.auto_update = true;
        else if (s == "-eval" && need(3)) {
            a.eval = true;
            a.t0 = (float)std::atof(argv[++i]); a.t1 = (float)std::atof(argv[++i]); a.n_eval = std::atoi(argv[++i]);
        } else if (pos == 0) { a.data = s; ++pos; }
        else if (pos == 1) { a.path = s; ++pos; }
        else if (pos == 2) { a.out_dir = s; ++pos; }
        else return false;
    }
    return a.eval ? !a.path.empty() || !a.data.empty() : pos == 3;
}

void usage()
{
    std::cout << "usage: render_path data camera_path.json output-dir [-frames N] [-spp N] [-r W H] [-cache] [-auto]"
                 " [-cache-r W H]\n       render_path camera_path.json -eval T0 T1 N\n";
}

void print_camera(float t, const fvc_path::CameraKeyFrame &k)
{
    const CameraMatrix m = k.m();
    std::cout << std::setprecision(9) << "{\"t\":" << t << ",\"cam2world\":[[" << m.m0.x << "," << m.m0.y << "," << m.m0.z << ","
              << m.m0.w << "],[" << m.m1.x << "," << m.m1.y << "," << m.m1.z << "," << m.m1.w << "],[" << m.m2.x << ","
              << m.m2.y << "," << m.m2.z << "," << m.m2.w << "]],\"R\":[" << k.R.w << "," << k.R.x << "," << k.R.y << ","
              << k.R.z << "],\"aperture_size\":" << k.aperture_size << ",\"focus_distance\":" << k.focus_distance << "}\n";
}

}  // namespace

int main(int argc, char **argv)
{
    Args a;
    if (!parse(argc, argv, a)) {
        usage();
        return 2;
    }
    fvc_path::CameraPath path;
    if (a.eval) {
        const std::string file = a.path.empty() ? a.data : a.path;
        if (!path.load(file)) { std::cerr << "cannot read " << file << "\n"; return 1; }
        for (int i = 0; i < a.n_eval; ++i) {
            const float t = a.n_eval > 1 ? a.t0 + (a.t1 - a.t0) * (float)i / (float)(a.n_eval - 1) : a.t0;
            print_camera(t, path.eval_camera_path(t));
        }
        return 0;
    }
    if (!path.load(a.path)) { std::cerr << "cannot read " << a.path << "\n"; return 1; }
    fvc_path::RenderSettings &rs = path.settings;
    if (a.res_w > 0) rs.resolution = make_int2(a.res_w, a.res_h);
    if (a.spp > 0) rs.spp = a.spp;
    if (a.cache) rs.render_from_cache = true;
    if (a.auto_update) rs.auto_cache_update = true;
    const uint32_t n_frames = a.frames >= 0 ? (uint32_t)a.frames : rs.n_frames();
    const int2 cache_res = a.cache_w > 0 ? make_int2(a.cache_w, a.cache_h) : rs.resolution;
    fs::create_directories(a.out_dir);

    LoaderData loader;
    if (!load_data(a.data, loader)) return 1;
    const SceneInfo scene_info = loader.scene_info;
    const StepsizeInfo stepsize = loader.stepsize_info;
    StepsizeInfo cache_stepsize = stepsize; /* m_cache_double_sampling_rate (application.h:87) */
    cache_stepsize.changeSamplingRate(2.0f, scene_info);

    CameraInfo cam{};
    cam.resolution = rs.resolution;
    cam.is_open_gl = false;
    const float focal_x = ((float)rs.resolution.x * 0.5f) / std::tan(rs.fov_x_deg * 0.5f * 3.14159265358979323846f / 180.f);
    cam.focal = make_float2(focal_x, focal_x);
    cam.principal = make_float2(rs.resolution.x * 0.5f, rs.resolution.y * 0.5f);

    CudaBuffer<uint8_t> &grid = loader.occupancy_grid_morton_bitfield;
    Cache cache_a, cache_b;
    PerformanceRenderer plain(scene_info, grid, loader.nerf_network);
    plain.resizeRenderbuffers(rs.resolution);
    CachePerformanceRenderer cached(scene_info, grid, loader.nerf_network, &cache_a, &cache_b);
    CacheSettings settings = CacheRenderer::default_cache_settings;
    settings.interpol_variant = loader.nerf_network.m_first_latent_is_density ? DensityIntermediates : Density;
    cached.setCacheSettings(settings);
    cached.resizeRenderbuffers(rs.resolution);
    if (rs.render_from_cache) {
        cached.resizeCache(cache_res, cache_stepsize);
        cached.swapCache();
        cached.resizeCache(cache_res, cache_stepsize);
    }
    ImageBuffer image(rs.resolution), debug(cache_res);

    float hit_ratio = 0.0f;
    float last_pos[3] = {1e30f, 1e30f, 1e30f};
    std::ofstream log(fs::path(a.out_dir) / "frames.json");
    log << "[";
    for (uint32_t f = 0; f < n_frames; ++f) {
        CameraInfo next = cam, cache_cam = cam;
        fvc_path::frame_cameras(path, f, cam, next, cache_cam);
        bool updated = false;
        float build_ms = 0.0f;
        if (fvc_path::needs_cache_update(rs, hit_ratio, cam.cam2world, last_pos)) {
            cache_cam.resize(cache_res);
            const RaymarchInfo cache_rm{cache_cam, {}, cache_stepsize, 0, false, true};
            const auto t0 = std::chrono::steady_clock::now();
            cached.initCacheBlockwise(cache_rm, debug);
            cached.swapCache();
            build_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
            last_pos[0] = cache_cam.cam2world.m0.w; last_pos[1] = cache_cam.cam2world.m1.w; last_pos[2] = cache_cam.cam2world.m2.w;
            updated = true;
        }
        RaymarchInfo rm{cam, next, stepsize, 0, true, false};
        const auto t0 = std::chrono::steady_clock::now();
        for (rm.sample_index = 0; rm.sample_index < rs.spp; ++rm.sample_index) {
            if (rs.render_from_cache) cached.render(rm, image);
            else plain.render(rm, image);
        }
        const float render_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        float spp_eval = 0.0f;
        if (rs.render_from_cache) {
            spp_eval = cached._render_stats.samples_ppx;
            hit_ratio = spp_eval > 0.0f ? cached._render_stats.cache_samples_evaluated / spp_eval : 0.0f;
        } else {
            spp_eval = plain._render_stats.samples_ppx;
        }
        std::ostringstream name;
        name << "frame_" << std::setfill('0') << std::setw(6) << f << ".png";
        image.writeToFile(fs::path(a.out_dir) / name.str());
        log << (f ? "," : "") << "\n{\"frame\":" << f << ",\"cache_update\":" << (updated ? "true" : "false")
            << ",\"cache_build_ms\":" << build_ms << ",\"hit_ratio\":" << hit_ratio << ",\"samples_ppx\":" << spp_eval
            << ",\"render_ms\":" << render_ms << ",\"spp\":" << rs.spp << ",\"cam_t\":[" << cam.cam2world.m0.w << ","
            << cam.cam2world.m1.w << "," << cam.cam2world.m2.w << "]}";
        std::cout << "Frame " << f << " | " << (updated ? "Cache Init | " : "") << "Render | Total: " << render_ms
                  << " Avg: " << render_ms / rs.spp << " SPP: " << rs.spp << std::endl;
    }
    log << "\n]\n";
    return 0;
}
