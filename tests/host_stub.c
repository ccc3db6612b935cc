/* A C host driving one frame through the C ABI, the way an engine's display() would (main.cpp:1077-1303 of
 * the reference): context, scene from an OBJ file, lights, camera, one frame into a device RGBA8 buffer,
 * read back. tests/test_abi.py compiles it as C99 and as C++17 and links it against librsh.so (it is not
 * run there: the CPU suite has no GPU). Usage: host_stub scene.obj out.png */
#include <stdio.h>
#include <stdlib.h>

#include "rsh.h"

#define CHECK(call)                                                                  \
    do {                                                                             \
        rsh_status st_ = (call);                                                     \
        if (st_ != RSH_OK) {                                                         \
            fprintf(stderr, "%s: %d (%s)\n", #call, (int)st_, rsh_last_error_string()); \
            return 1;                                                                \
        }                                                                            \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const uint32_t W = 640, H = 360, depth = 2;
    rsh_config cfg;
    rsh_config_default(&cfg);
    cfg.flags |= RSH_FLAG_FUSED;  /* the batched form; 0 keeps the plain stage-by-stage path */
    rsh_ctx* ctx = NULL;
    CHECK(rsh_create(&cfg, &ctx));
    rsh_obj_data* obj = NULL;
    CHECK(rsh_obj_load(argv[1], &obj));
    rsh_scene* scene = NULL;
    CHECK(rsh_scene_upload(ctx, &obj->desc, &scene));
    rsh_obj_free(obj);
    float lo[3], hi[3];
    CHECK(rsh_scene_bounds(scene, lo, hi));
    rsh_light light = {{0.5f * (lo[0] + hi[0]), hi[1], 0.5f * (lo[2] + hi[2])}, {1.f, 1.f, 1.f}, 1.f, 1.f};
    CHECK(rsh_lights_set(ctx, &light, 1));
    /* eye in front of the box, looking down -z; direction scaled by the view distance, right/up by the
     * half extents of the image plane (Camera.cpp:91-133) */
    const float dist = 2.0f * (hi[2] - lo[2]) + 1.0f;
    rsh_camera cam = {{0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), hi[2] + dist},
                      {0.f, 0.f, -dist},
                      {dist * 1.1547f * (float)W / (float)H, 0.f, 0.f},
                      {0.f, dist * 1.1547f, 0.f}};
    CHECK(rsh_camera_set(ctx, &cam));
    rsh_stream_t stream = NULL;
    CHECK(rsh_stream_create(&stream));
    uint32_t* rgba_dev = NULL;
    CHECK(rsh_malloc((void**)&rgba_dev, 4ull * W * H));
    CHECK(rsh_render_frame(ctx, scene, W, H, depth, rgba_dev, stream));
    uint32_t* rgba = (uint32_t*)malloc(4ull * W * H);
    if (!rgba) return 1;
    CHECK(rsh_memcpy_d2h(rgba, rgba_dev, 4ull * W * H, stream));
    CHECK(rsh_stream_synchronize(stream));
    CHECK(rsh_check_device_errors(ctx, stream));
    CHECK(rsh_write_png(argv[2], rgba, W, H));
    free(rgba);
    CHECK(rsh_free(rgba_dev));
    CHECK(rsh_stream_destroy(stream));
    CHECK(rsh_scene_destroy(ctx, scene));
    CHECK(rsh_destroy(ctx));
    return 0;
}
