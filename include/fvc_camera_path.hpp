/*
 * fvc_camera_path.hpp - the real-time viewer's key-framed camera path
 * (realtime_viewer/include/camera_path.h, realtime_viewer/src/camera_path.cu)
 * and its cache-update rule (realtime_viewer/src/application.cu:132-158,
 * 248-312), header-only C++ over fvc.hpp.
 *
 *   CameraKeyFrame  rotation quaternion R, translation T, aperture size and
 *                   focus distance of one key frame (camera_path.h:17-41)
 *   spline          centripetal-free Catmull-Rom through four key frames as
 *                   three levels of key-frame lerps (slerp on R, linear on
 *                   the rest), the construction of instant-ngp's camera path
 *                   that the viewer follows (camera_path.cu:14-48)
 *   CameraPath      the key frames, the render settings and
 *                   eval_camera_path(t), t in [0, 1] over all key frames with
 *                   the end frames repeated (camera_path.h:44-103); load/save
 *                   of the viewer's JSON ({"settings": {...}, "path":
 *                   [{"R", "T", "aperture_size", "focus_distance"}]})
 *   needs_cache_update  the path renderer's rule: rebuild when the path does
 *                   not update automatically, or when the last frame's cache
 *                   hit ratio fell below the limit, or when the camera moved
 *                   farther than the update distance from the last build
 *   frame_cameras   the cameras of path frame i: the frame's camera, the next
 *                   frame's camera (the motion-blur end pose) and the cache
 *                   camera half a frame ahead
 *
 * Quaternion arithmetic is fvc_sampling.h's (the same slerp the motion blur
 * uses).  JSON: R is stored as [x, y, z, w], the order of tiny-cuda-nn's
 * vec_json serialiser that the viewer's files go through (tiny-cuda-nn is a
 * dependency the reference tree does not vendor).
 */
#pragma once

#include "fvc.hpp"
#include "../frustumvolumecaching_gb300/csrc/fvc_sampling.h"

#include <fstream>
#include <sstream>

namespace fvc_path {

using fvc_smp::Quat;

struct CameraKeyFrame {
    Quat R{1.0f, 0.0f, 0.0f, 0.0f};
    float T[3] = {0.0f, 0.0f, 0.0f};
    float aperture_size = 0.0f;
    float focus_distance = 1.0f;

    CameraKeyFrame() = default;
    /* from a camera: the rotation block's quaternion and the translation column */
    CameraKeyFrame(const CameraMatrix &cam, float ap, float fd) : aperture_size(ap), focus_distance(fd)
    {
        const float m[12] = {cam.m0.x, cam.m0.y, cam.m0.z, cam.m0.w, cam.m1.x, cam.m1.y, cam.m1.z, cam.m1.w,
                             cam.m2.x, cam.m2.y, cam.m2.z, cam.m2.w};
        R = fvc_smp::quat_from(m);
        T[0] = cam.m0.w; T[1] = cam.m1.w; T[2] = cam.m2.w;
    }
    /* the camera matrix of the normalised rotation and the translation */
    CameraMatrix m() const
    {
        const Quat q = fvc_smp::qnormalize(R);
        const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z, xz = q.x * q.z, xy = q.x * q.y, yz = q.y * q.z;
        const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
        CameraMatrix c;
        c.m0 = make_float4(1.0f - 2.0f * (yy + zz), 2.0f * (xy - wz), 2.0f * (xz + wy), T[0]);
        c.m1 = make_float4(2.0f * (xy + wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz - wx), T[1]);
        c.m2 = make_float4(2.0f * (xz - wy), 2.0f * (yz + wx), 1.0f - 2.0f * (xx + yy), T[2]);
        return c;
    }
};

/* key-frame lerp over the parameter interval [t0, t1]: slerp on the short arc,
 * the rest linear (camera_path.cu:14-29) */
inline CameraKeyFrame lerp(const CameraKeyFrame &p0, const CameraKeyFrame &p1, float t, float t0, float t1)
{
    t = (t - t0) / (t1 - t0);
    Quat R1 = p1.R;
    if (fvc_smp::qdot(R1, p0.R) < 0.0f) R1 = {-R1.w, -R1.x, -R1.y, -R1.z};
    CameraKeyFrame r;
    r.R = fvc_smp::qnormalize(fvc_smp::qslerp(p0.R, R1, t));
    for (int k = 0; k < 3; ++k) r.T[k] = p0.T[k] + (p1.T[k] - p0.T[k]) * t;
    r.aperture_size = p0.aperture_size + (p1.aperture_size - p0.aperture_size) * t;
    r.focus_distance = p0.focus_distance + (p1.focus_distance - p0.focus_distance) * t;
    return r;
}

/* Catmull-Rom between p1 and p2 at t in [0, 1] (camera_path.cu:40-48) */
inline CameraKeyFrame spline(float t, const CameraKeyFrame &p0, const CameraKeyFrame &p1, const CameraKeyFrame &p2,
                             const CameraKeyFrame &p3)
{
    const CameraKeyFrame q0 = lerp(p0, p1, t, -1.0f, 0.0f);
    const CameraKeyFrame q1 = lerp(p1, p2, t, 0.0f, 1.0f);
    const CameraKeyFrame q2 = lerp(p2, p3, t, 1.0f, 2.0f);
    const CameraKeyFrame r0 = lerp(q0, q1, t, -1.0f, 1.0f);
    const CameraKeyFrame r1 = lerp(q1, q2, t, 0.0f, 2.0f);
    return lerp(r0, r1, t, 0.0f, 1.0f);
}

struct RenderSettings { /* CameraPath::RenderSettings, camera_path.h:47-75 */
    bool render_from_cache = false;
    bool auto_cache_update = false;
    float cache_update_distance = 1.1f;
    float cache_hit_limit = 0.5f;
    int2 resolution = {1920, 1080};
    float fov_x_deg = 60.0f;
    int spp = 8;
    float fps = 60.0f;
    float duration_seconds = 5.0f;
    float shutter_fraction = 0.5f;
    int quality = 10;
    uint32_t n_frames() const { return (uint32_t)((double)duration_seconds * fps); }
};

struct CameraPath {
    std::vector<CameraKeyFrame> key_frames;
    RenderSettings settings;

    const CameraKeyFrame &get_keyframe(int i) const
    {
        return key_frames[std::min(std::max(i, 0), (int)key_frames.size() - 1)];
    }
    /* t in [0, 1] across the key frames (camera_path.h:91-99) */
    CameraKeyFrame eval_camera_path(float t) const
    {
        if (key_frames.empty()) return {};
        t *= (float)key_frames.size() - 1;
        const int t1 = (int)std::floor(t);
        return spline(t - std::floor(t), get_keyframe(t1 - 1), get_keyframe(t1), get_keyframe(t1 + 1), get_keyframe(t1 + 2));
    }

    bool load(const fs::path &path)
    {
        std::ifstream f(path);
        if (!f) return false;
        const fvc_cpp::Json j = fvc_cpp::read_json(path);
        key_frames.clear();
        if (j.contains("settings")) {
            const fvc_cpp::Json &s = j["settings"];
            settings.resolution = make_int2((int)s["resolution"][0].f(), (int)s["resolution"][1].f());
            settings.render_from_cache = s["render_from_cache"].b;
            settings.auto_cache_update = s["auto_cache_update"].b;
            settings.cache_update_distance = (float)s["cache_update_distance"].f();
            settings.cache_hit_limit = (float)s["cache_min_hit_ratio"].f();
            settings.fov_x_deg = (float)s["fov_x"].f();
            settings.spp = (int)s["spp"].f();
            settings.fps = (float)s["fps"].f();
            settings.duration_seconds = (float)s["duration"].f();
            settings.shutter_fraction = (float)s["shutter_fraction"].f();
            settings.quality = (int)s["quality"].f();
        }
        if (j.contains("path")) {
            for (const fvc_cpp::Json &e : j["path"].arr) {
                CameraKeyFrame k;
                const fvc_cpp::Json &R = e["R"];
                k.R = {(float)R[3].f(), (float)R[0].f(), (float)R[1].f(), (float)R[2].f()};
                for (int c = 0; c < 3; ++c) k.T[c] = (float)e["T"][c].f();
                k.aperture_size = (float)e["aperture_size"].f();
                k.focus_distance = (float)e["focus_distance"].f();
                key_frames.push_back(k);
            }
        }
        return true;
    }

    void save(const fs::path &path) const
    {
        std::ostringstream o;
        o.precision(9);
        const RenderSettings &s = settings;
        o << "{\"settings\":{\"resolution\":[" << s.resolution.x << "," << s.resolution.y << "],\"fov_x\":" << s.fov_x_deg
          << ",\"render_from_cache\":" << (s.render_from_cache ? "true" : "false")
          << ",\"auto_cache_update\":" << (s.auto_cache_update ? "true" : "false")
          << ",\"cache_update_distance\":" << s.cache_update_distance << ",\"cache_min_hit_ratio\":" << s.cache_hit_limit
          << ",\"spp\":" << s.spp << ",\"fps\":" << s.fps << ",\"duration\":" << s.duration_seconds
          << ",\"shutter_fraction\":" << s.shutter_fraction << ",\"quality\":" << s.quality << "},\"path\":[";
        for (size_t i = 0; i < key_frames.size(); ++i) {
            const CameraKeyFrame &k = key_frames[i];
            o << (i ? "," : "") << "{\"R\":[" << k.R.x << "," << k.R.y << "," << k.R.z << "," << k.R.w << "],\"T\":[" << k.T[0]
              << "," << k.T[1] << "," << k.T[2] << "],\"aperture_size\":" << k.aperture_size
              << ",\"focus_distance\":" << k.focus_distance << "}";
        }
        o << "]}";
        std::ofstream f(path);
        f << o.str();
    }
};

/* Application::setCameraFromKeyFrame (application.cu:338-344) */
inline void set_camera_from_keyframe(const CameraKeyFrame &f, CameraInfo &cam)
{
    cam.cam2world = f.m();
    cam.world2cam = cam.cam2world.inverse();
    cam.aperature = f.aperture_size;
    cam.focus_z = f.focus_distance;
}

/* the path renderer's cache-update rule (application.cu:276-277) */
inline bool needs_cache_update(const RenderSettings &s, float last_hit_ratio, const CameraMatrix &cam, const float *last_build_pos)
{
    if (!s.render_from_cache) return false;
    if (!s.auto_cache_update) return true;
    const float dx = cam.m0.w - last_build_pos[0], dy = cam.m1.w - last_build_pos[1], dz = cam.m2.w - last_build_pos[2];
    return last_hit_ratio < s.cache_hit_limit || std::sqrt(dx * dx + dy * dy + dz * dz) > s.cache_update_distance;
}

/* the cameras of path frame i of n (application.cu:269-274, 137-142):
 * play time i / n, the next frame's pose 1 / n later (motion blur) and the
 * cache pose half a frame ahead */
inline void frame_cameras(const CameraPath &p, uint32_t i, CameraInfo &cam, CameraInfo &next, CameraInfo &cache_cam)
{
    const uint32_t n = std::max(1u, p.settings.n_frames());
    const float play = (float)((double)i / (double)n);
    set_camera_from_keyframe(p.eval_camera_path(play), cam);
    next = cam;
    set_camera_from_keyframe(p.eval_camera_path(play + 1.0f / n), next);
    cache_cam = cam;
    set_camera_from_keyframe(p.eval_camera_path(play + 0.5f / n), cache_cam);
}

}  // namespace fvc_path
