/* A plain C caller of the library (C99, no C++): includes every public C
 * header, links against libpyrsgm_gb300.so and exercises calls that need no
 * GPU -- argument rejection, parameter validation, level geometry, the
 * kernel-form switches, file I/O and metrics.  Prints "ok" and exits 0 when every check holds. */
#include <stdio.h>
#include <string.h>

#include <pyrsgm/pyrsgm_c.h>
#include <pyrsgm/pyrsgm_gb300.h>
#include <pyrsgm/pyrsgm_io.h>
#include <pyrsgm/pyrsgm_tri3sgm.h>

static int fails = 0;
#define CHECK(c)                                                \
    do {                                                        \
        if (!(c)) {                                             \
            fprintf(stderr, "line %d: %s\n", __LINE__, #c);     \
            ++fails;                                            \
        }                                                       \
    } while (0)

int main(int argc, char** argv)
{
    char err[256];
    /* the reference's C API: wrong pyrDown size, bad label counts */
    CHECK(pyrsgm_pyrdown_u8((const unsigned char*)1, 64, 64, 48, (unsigned char*)2, 32, 31, 24, 0) == -1);
    void* ws = pyrsgm_create_workspace();
    CHECK(ws != NULL);
    CHECK(pyrsgm_workspace_reserve(ws, 64, 48, 24) == -1);
    CHECK(pyrsgm_workspace_reserve(NULL, 64, 48, 32) == -1);
    CHECK(pyrsgm_compute_single_scale(ws, NULL, (const unsigned char*)2, NULL, NULL, NULL, 64, 64, 128, 256, 256, 64,
                                      48, 32, 0, 5, 8, 32, 10, 1, 63, PYRSGM_COST_CENSUS, PYRSGM_POST_LRCHECK, 3, 0,
                                      1.0f, 1.0f, 1.0f, 1.0f, 0) == -1);
    /* the Tri3SGM names reject the same way */
    CHECK(cuda_3sgm_compute_with_workspace(ws, NULL, (const unsigned char*)2, NULL, NULL, NULL, 64, 64, 128, 256,
                                           256, 64, 48, 32, 0, 5, 8, 32, 10, 1, 63, PYRSGM_COST_CENSUS,
                                           PYRSGM_POST_LRCHECK, 3, 0, 1.0f, 1.0f, 1.0f, 1.0f, 0) == -1);
    pyrsgm_destroy_workspace(ws);

    /* Params through C: defaults, validation, level geometry */
    pyrsgm_gb300_params p, v;
    pyrsgm_gb300_default_params(&p);
    p.num_disparities = 256;
    p.pyramid_levels = 3;
    CHECK(pyrsgm_gb300_validate_params(&p, &v, err, sizeof err) == 0);
    int geo[35];
    CHECK(pyrsgm_gb300_level_geometry(1920, 1080, &p, geo, err, sizeof err) == 4);
    CHECK(geo[1] == 1920 && geo[2] == 1080 && geo[3] == 16);   /* level 0: width, height, 16 local labels */
    p.pyramid_levels = 9;
    CHECK(pyrsgm_gb300_validate_params(&p, &v, err, sizeof err) == -1 && strstr(err, "pyramid_levels"));

    /* PGM round trip and metrics (host only) */
    if (argc > 1) {
        unsigned char img[12] = {0, 10, 20, 30, 40, 50, 60, 70, 80, 90, 100, 110}, back[12];
        int w = 0, h = 0;
        CHECK(pyrsgm_gb300_write_pgm(argv[1], img, 4, 4, 3, err, sizeof err) == 0);
        CHECK(pyrsgm_gb300_read_pgm(argv[1], NULL, 0, &w, &h, err, sizeof err) == 0 && w == 4 && h == 3);
        CHECK(pyrsgm_gb300_read_pgm(argv[1], back, 4, &w, &h, err, sizeof err) == 0 &&
              memcmp(img, back, sizeof img) == 0);
    }
    /* kernel-form switches and the checked-build report (host state only) */
    int prev = pyrsgm_gb300_set_tbw(2);
    CHECK(pyrsgm_gb300_set_tbw(prev) == 2);
    CHECK(pyrsgm_gb300_set_tbw(3) == -1);
    CHECK(pyrsgm_gb300_checked() == 0);
    CHECK(pyrsgm_gb300_check_report(err, sizeof err) == 0 && err[0] == 0);

    float d[4] = {1.0f, 2.0f, 0.0f, 4.5f}, g[4] = {1.0f, 4.0f, 3.0f, 4.0f};
    pyrsgm_gb300_metrics m;
    CHECK(pyrsgm_gb300_evaluate(d, 4, g, 4, NULL, 0, 4, 1, 100.0f, &m) == 0);
    CHECK(m.evaluated == 4 && m.valid == 3);
    if (fails == 0) printf("ok\n");
    return fails == 0 ? 0 : 1;
}
