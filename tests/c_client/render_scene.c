/* A C client of libatx.so: loads a scene file in the reference's format,
 * renders it and writes the image, the way Ataraxia's ImportScene + Render +
 * display sequence (Engine/src/main.cpp:196-217) uses the library.
 *
 *   render_scene SCENE.json OUT.ppm WIDTH HEIGHT SPP
 *
 * Prints the frame index reached and a checksum of the RGBA8 image. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "atx.h"

static int check(atx_status s, const char* what)
{
    if (s == ATX_OK) return 0;
    fprintf(stderr, "%s: %s: %s\n", what, atx_status_string(s), atx_last_error());
    return 1;
}

int main(int argc, char** argv)
{
    if (argc != 6) {
        fprintf(stderr, "usage: %s SCENE.json OUT.ppm WIDTH HEIGHT SPP\n", argv[0]);
        return 2;
    }
    const uint32_t w = (uint32_t)strtoul(argv[3], NULL, 10), h = (uint32_t)strtoul(argv[4], NULL, 10);
    const uint32_t spp = (uint32_t)strtoul(argv[5], NULL, 10);
    atx_scene* scene = NULL;
    atx_renderer* r = NULL;
    atx_scene_info info;
    uint32_t frame = 0;
    int rc = 1;
    if (check(atx_scene_load(argv[1], &scene), "load")) return 1;
    if (check(atx_scene_get_info(scene, &info), "info")) goto out;
    if (check(atx_renderer_create(NULL, &r), "create")) goto out;
    if (check(atx_resize(r, w, h), "resize")) goto out;
    if (check(atx_set_scene_graph(r, scene), "scene")) goto out;
    if (check(atx_set_settings(r, &info.settings), "settings")) goto out;
    if (check(atx_set_camera(r, &info.camera), "camera")) goto out;
    if (check(atx_render(r, spp), "render")) goto out;
    if (check(atx_save_image(r, argv[2], ATX_IMAGE_PPM), "save")) goto out;
    if (check(atx_get_frame_index(r, &frame), "frame")) goto out;
    {
        const uint64_t n = (uint64_t)w * h;
        uint32_t* img = (uint32_t*)malloc(n * sizeof(uint32_t));
        uint64_t sum = 0;
        if (!img) goto out;
        if (check(atx_read_image(r, img, n), "read")) {
            free(img);
            goto out;
        }
        for (uint64_t i = 0; i < n; ++i) sum = sum * 1000003u + img[i];
        free(img);
        printf("frame %u checksum %016llx\n", frame, (unsigned long long)sum);
    }
    rc = 0;
out:
    if (r) atx_renderer_destroy(r);
    if (scene) atx_scene_destroy(scene);
    return rc;
}
