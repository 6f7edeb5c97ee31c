/*
 * A plain C99 client of the library's C ABI (include/gs300.h), compiled and run by
 * tests/test_c_abi.py.  It shows that the public header is C (no CUDA or C++ types) and that a
 * program in another language can link the shared library and drive it.
 *
 *   gs_abi_smoke host              prints host-side results (no device work)
 *   gs_abi_smoke render IN OUT W H renders the gs_gaussian_pod records in file IN through the
 *                                  Viewer facade with an orbit camera and writes the RGBA8
 *                                  frame (W*H*4 bytes) to file OUT
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gs300.h"

static int fail(const char *what, gs_status s) {
    fprintf(stderr, "%s failed: status %d: %s\n", what, (int)s, gs_last_error());
    return 1;
}

static void print_bits(const char *name, const float *v, int n) {
    int i;
    printf("%s", name);
    for (i = 0; i < n; ++i) {
        uint32_t b;
        memcpy(&b, &v[i], 4);
        printf(" %08x", (unsigned)b);
    }
    printf("\n");
}

static gs_camera orbit_camera(void) {
    gs_camera c;
    c.z_near = 0.1f;
    c.z_far = 1e4f;
    c.vertical_fov = (float)(60.0 * 3.14159265358979323846 / 180.0);
    c.pitch = 0.1f;
    c.yaw = 0.1f;
    c.pos[0] = -6.0f * sinf(c.yaw) * cosf(c.pitch);
    c.pos[1] = -6.0f * sinf(c.pitch);
    c.pos[2] = -6.0f * cosf(c.yaw) * cosf(c.pitch);
    return c;
}

static int host(void) {
    gs_camera c = orbit_camera();
    gs_camera_pod pod;
    gs_gaussian_transform_pod gt;
    gs_status s;
    printf("version %s\n", gs_version());
    printf("depth_capacity %u %u %u\n", (unsigned)gs_depth_capacity(0), (unsigned)gs_depth_capacity(1000000),
           (unsigned)gs_depth_capacity(3840));
    s = gs_camera_pod_new(&c, 1920, 1080, &pod);
    if (s != GS_OK) return fail("gs_camera_pod_new", s);
    print_bits("camera", c.pos, 3);
    print_bits("view", pod.view, 16);
    print_bits("proj", pod.proj, 16);
    print_bits("size", pod.size, 2);
    s = gs_gaussian_transform_pod_new(1.0f, GS_DISPLAY_SPLAT, 4, 0, 3.0f, &gt);
    printf("bad_sh_degree %d\n", (int)s);
    printf("sizeof %u %u %u\n", (unsigned)sizeof(gs_gaussian_pod), (unsigned)sizeof(gs_camera_pod),
           (unsigned)sizeof(gs_frame_uniforms));
    return 0;
}

static int render(const char *in, const char *out, uint32_t w, uint32_t h) {
    FILE *f = fopen(in, "rb");
    long bytes;
    void *records;
    uint32_t n;
    gs_viewer *v = NULL;
    gs_target *t = NULL;
    gs_camera c = orbit_camera();
    uint8_t *frame;
    gs_status s;
    if (!f) return 1;
    fseek(f, 0, SEEK_END);
    bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    records = malloc((size_t)bytes);
    if (!records || fread(records, 1, (size_t)bytes, f) != (size_t)bytes) return 1;
    fclose(f);
    n = (uint32_t)(bytes / (long)sizeof(gs_gaussian_pod));
    if ((s = gs_viewer_create(records, n, GS_FORMAT_FP32, &v)) != GS_OK) return fail("gs_viewer_create", s);
    if ((s = gs_viewer_update_camera(v, &c, w, h)) != GS_OK) return fail("gs_viewer_update_camera", s);
    if ((s = gs_target_create(w, h, &t)) != GS_OK) return fail("gs_target_create", s);
    if ((s = gs_viewer_render(v, gs_target_data(t), w, h, gs_target_pitch(t), NULL)) != GS_OK)
        return fail("gs_viewer_render", s);
    if ((s = gs_viewer_synchronize(v, NULL)) != GS_OK) return fail("gs_viewer_synchronize", s);
    frame = (uint8_t *)malloc((size_t)w * h * 4);
    if (!frame) return 1;
    if ((s = gs_target_download(t, frame, NULL)) != GS_OK) return fail("gs_target_download", s);
    f = fopen(out, "wb");
    if (!f || fwrite(frame, 1, (size_t)w * h * 4, f) != (size_t)w * h * 4) return 1;
    fclose(f);
    printf("rendered %u gaussians %ux%u\n", (unsigned)n, (unsigned)w, (unsigned)h);
    gs_target_destroy(t);
    gs_viewer_destroy(v);
    free(frame);
    free(records);
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 2 && strcmp(argv[1], "host") == 0) return host();
    if (argc >= 6 && strcmp(argv[1], "render") == 0)
        return render(argv[2], argv[3], (uint32_t)atoi(argv[4]), (uint32_t)atoi(argv[5]));
    fprintf(stderr, "usage: %s host | render IN OUT W H\n", argv[0]);
    return 2;
}
