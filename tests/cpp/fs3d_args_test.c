/* fs3d_args_test.c — include/fs3d.h from plain C (C11): the 3D entry points
 * link, and arguments are checked before any device work, so this runs on a
 * machine without a GPU.  Prints OK on success. */
#include <stdio.h>
#include <string.h>

#include "fs2d.h"
#include "fs3d.h"

static int expect(int got, int want, const char* what) {
    if (got != want) {
        printf("FAIL %s: %d (expected %d): %s\n", what, got, want, fs2d_last_error());
        return 1;
    }
    return 0;
}

int main(void) {
    int bad = 0;
    double result = 7.0;
    fs3d_array a = {NULL, 2, 3, 4};
    fs3d_array wrong = {NULL, 2, 3, 5};
    fs3d_array empty = {NULL, 0, 3, 4};
    fs3d_mac g;
    memset(&g, 0, sizeof(g));
    g.sizeX = 3;
    g.sizeY = 2;
    g.sizeZ = 2;
    g.u = (fs3d_array){NULL, 4, 2, 2};
    g.v = (fs3d_array){NULL, 3, 3, 2};
    g.w = (fs3d_array){NULL, 3, 2, 3};
    bad |= expect(fs3d_add(NULL, &a, NULL), FS2D_ERR_INVALID, "add NULL");
    bad |= expect(fs3d_add(&wrong, &a, NULL), FS2D_ERR_INVALID, "add extents");
    bad |= expect(fs3d_set_multiply_add(&a, &a, 1.0, &wrong, NULL), FS2D_ERR_INVALID, "setMultiplyAdd extents");
    bad |= expect(fs3d_inner_product(&a, &a, NULL, NULL), FS2D_ERR_INVALID, "innerProduct NULL result");
    bad |= expect(fs3d_infinite_norm(&a, NULL, NULL), FS2D_ERR_INVALID, "infiniteNorm NULL result");
    bad |= expect(fs3d_mac_face_vel(&g, 7, NULL, NULL), FS2D_ERR_INVALID, "faceVel axis");
    bad |= expect(fs3d_mac_vel_interp(&g, FS3D_UVW + 1, NULL, 1, NULL, NULL), FS2D_ERR_INVALID, "velInterp component");
    g.v.NY = 2;
    bad |= expect(fs3d_mac_vel_div(&g, NULL, NULL), FS2D_ERR_INVALID, "velDiv face extents");
    /* empty arrays and point sets need no device */
    bad |= expect(fs3d_add(&empty, &empty, NULL), FS2D_OK, "add empty");
    bad |= expect(fs3d_inner_product(&empty, &empty, &result, NULL), FS2D_OK, "innerProduct empty");
    if (result != 0.0) {
        printf("FAIL innerProduct of an empty array is %g\n", result);
        bad = 1;
    }
    bad |= expect(fs3d_tricubic(&a, NULL, 0, NULL, NULL), FS2D_OK, "triCubic no points");
    printf(bad ? "FAIL\n" : "OK\n");
    return bad;
}
