/*
 * Host-only checks of the C++ renderer API header (no GPU needed): the
 * reference's type layouts, the camera-file loader, the rigid inverse, the
 * field-of-view-keeping resize and the PNG writer.  Prints one line per check
 * and exits non-zero on the first failure.
 *
 *   api_check <nerfacc camera file> <png output path>
 */
#include "fvc.hpp"

#include <cassert>

static int fails = 0;
#define CHECK(c)                                                  \
    do {                                                          \
        if (!(c)) {                                               \
            std::cout << "FAIL " << #c << std::endl;              \
            ++fails;                                              \
        } else {                                                  \
            std::cout << "ok   " << #c << std::endl;              \
        }                                                         \
    } while (0)

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    CHECK(sizeof(SceneInfo) == 76 && sizeof(StepsizeInfo) == 48 && sizeof(CameraInfo) == 144 && sizeof(RaymarchInfo) == 352);
    CHECK(offsetof(RaymarchInfo, sample_index) == 336 && offsetof(CameraInfo, world2cam) == 80);

    CameraInfo ci{};
    std::vector<CameraPathDataEntry> path;
    CHECK(load_camerapath(argv[1], NERFACC, ci, path));
    CHECK(path.size() == 2);
    CHECK(ci.resolution.x == 40 && ci.resolution.y == 30 && !ci.is_open_gl);
    CHECK(std::fabs(ci.principal.x - 20.0f) < 1e-6f && std::fabs(ci.principal.y - 15.0f) < 1e-6f);
    CHECK(path[1].image_path.extension() == ".png");

    /* the inverse of a rigid transform composes to the identity */
    const CameraMatrix m = path[0].transform_matrix, inv = m.inverse();
    const float4 r[3] = {m.m0, m.m1, m.m2}, q[3] = {inv.m0, inv.m1, inv.m2};
    float err = 0.0f;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 4; ++j) {
            const float qi[4] = {q[i].x, q[i].y, q[i].z, q[i].w};
            const float col[4] = {j == 0 ? r[0].x : j == 1 ? r[0].y : j == 2 ? r[0].z : r[0].w,
                                  j == 0 ? r[1].x : j == 1 ? r[1].y : j == 2 ? r[1].z : r[1].w,
                                  j == 0 ? r[2].x : j == 1 ? r[2].y : j == 2 ? r[2].z : r[2].w, j == 3 ? 1.0f : 0.0f};
            float v = 0.0f;
            for (int k = 0; k < 4; ++k) v += qi[k] * col[k];
            err = std::max(err, std::fabs(v - (i == j ? 1.0f : 0.0f)));
        }
    CHECK(err < 1e-5f);

    CameraInfo big = ci;
    big.resize(make_int2(80, 60));
    CHECK(std::fabs(big.focal.y - 2.0f * ci.focal.y) < 1e-4f && big.principal.x == 40.0f);

    /* StepsizeInfo::setAdditionalInfo / changeSamplingRate (host only, through the library) */
    SceneInfo sc{};
    sc.grid_resolution = 128;
    sc.grid_nlvl = 1;
    sc.aabb_from = make_float3(-1.5f, -1.5f, -1.5f);
    sc.aabb_to = make_float3(1.5f, 1.5f, 1.5f);
    StepsizeInfo st{};
    st.cone_angle = 1.0f / 256.0f;
    st.stepsize = 0.002f;
    st.near = 0.0f;
    st.far = 1e10f;
    st.setAdditionalInfo(sc);
    StepsizeInfo half = st;
    half.changeSamplingRate(2.0f, sc);
    CHECK(st.dt_min == st.stepsize && st.i_max > st.i_min && st.t_max > st.t_min);
    CHECK(half.stepsize == st.stepsize / 2.0f && half.dt_min == half.stepsize && half.i_max > st.i_max);
    void (CacheRenderer::*fill)(RaymarchInfo, RenderBuffer &) = &CacheRenderer::initCache;
    CHECK(fill != nullptr);
    void (CacheBasicRenderer::*post)(RaymarchInfo, RenderBuffer &) = &CacheBasicRenderer::postRender;
    CHECK(post != nullptr);

    std::vector<uint8_t> px(7 * 5 * 4);
    for (size_t i = 0; i < px.size(); ++i) px[i] = (uint8_t)(i * 37);
    CHECK(fvc_cpp::write_png(argv[2], px.data(), 7, 5));

    fvc_cpp::Json j;
    const char *s = "{\"a\": [1, 2.5, -3e2], \"b\": {\"c\": true, \"d\": \"x\\\"y\"}, \"e\": null}";
    const char *p = s;
    j = fvc_cpp::parse_json(p, s + std::strlen(s));
    CHECK(j["a"][2].f() == -300.0f && j["b"]["c"].b && j["b"]["d"].str == "x\"y" && j["e"].kind == fvc_cpp::Json::NUL);
    std::cout << (fails ? "FAILED" : "PASSED") << std::endl;
    return fails ? 1 : 0;
}
