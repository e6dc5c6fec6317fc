/* The oracle: a scalar CPU restatement of the reference's Kerr hole trace, for the tests and the CPU
 * baseline only.  It is test infrastructure: the product (artful_gb300/) never links or calls it.
 *
 * It follows eugeniobenfica/artful v0.4.0 src/software/lens.inc (lensTrace 99-351, lensTile 355-383 and
 * the helpers 29-96), one ray at a time instead of eight lanes, with the same IEEE single-precision
 * operations in the same order (built with -ffp-contract=off).  Its FP32 results are pinned bit for
 * bit against the reference itself, built from its sources into oracle/_ref, and against the golden
 * fixtures in tests/golden/ made from it.  The FP64 instantiation evaluates the same formulas in
 * double from a frame computed in double: the check for the FP64 and mixed-precision GPU traces. */
#ifndef ARTF_ORACLE_H
#define ARTF_ORACLE_H

#include <stdint.h>

/* The frame block, laid out as the reference's ArtfHoleFrame (src/scene/sceneInternal.h:302-319). */
typedef struct OracleFrame {
    float er[4], etheta[4], ephi[4], right[4], up[4], forward[4], metric[4], place[4], spin[4], flow[4], boost[4],
        disc[4], look[4], image[4];
    uint32_t size[4];
    uint32_t bloom[8][4];
} OracleFrame;

/* The same fields in double (the FP64 frame). */
typedef struct OracleFrame64 {
    double er[4], etheta[4], ephi[4], right[4], up[4], forward[4], metric[4], place[4], spin[4], flow[4], boost[4],
        disc[4], look[4], image[4];
} OracleFrame64;

/* Where a ray ended, as the GPU trace's ArtfCudaRayEnd records it. */
typedef struct OracleEnd {
    float hitR, hitPhi, dir[3], mino;
    uint16_t steps;
    uint8_t crossings, kind;
    uint16_t fp64Steps, reserved; /* (always 0 here: the GPU's mixed trace counts its FP64 steps) */
} OracleEnd;

enum { ORACLE_HORIZON = 0, ORACLE_SKY = 1, ORACLE_OPAQUE = 2, ORACLE_CAP = 3, ORACLE_LIT = 0x10 };

/* Map layout (src/scene/sceneInternal.h:18-32, 324-329). */
#define ORACLE_MAP_WIDTH 2048
#define ORACLE_MAP_HEIGHT 1024
#define ORACLE_DUST_WIDTH 1024
#define ORACLE_DUST_HEIGHT 256
#define ORACLE_FLUID_WIDTH 1024
#define ORACLE_FLUID_HEIGHT 256
#define ORACLE_COLORS 256
#define ORACLE_SKY_WIDTH 1024
#define ORACLE_SKY_HEIGHT 512
#define ORACLE_ROWS_AT (ORACLE_MAP_WIDTH * ORACLE_MAP_HEIGHT)
#define ORACLE_COLORS_AT (ORACLE_ROWS_AT + ORACLE_MAP_HEIGHT * 2)
#define ORACLE_SKY_AT (ORACLE_COLORS_AT + ORACLE_COLORS * 3)
#define ORACLE_GLOW_AT (ORACLE_SKY_AT + ORACLE_SKY_WIDTH * ORACLE_SKY_HEIGHT)
#define ORACLE_DUST_AT (ORACLE_GLOW_AT + ORACLE_MAP_HEIGHT)
#define ORACLE_MAP_FLOATS (ORACLE_DUST_AT + ORACLE_DUST_WIDTH * ORACLE_DUST_HEIGHT)

/* Options of a trace: stepScale 1 is the reference's step (0.5 halves it and doubles the cap). */
typedef struct OracleOptions {
    float stepScale;
} OracleOptions;

/* n rays at image positions nx, ny (-1..1) and moments time[]: rgb (3 floats a ray); ends may be NULL. */
void oracleTrace32(const OracleFrame* h, const float* map, const float* fluid, const OracleOptions* o, int n,
                   const float* nx, const float* ny, const float* time, float* rgb, OracleEnd* ends);
void oracleTrace64(const OracleFrame64* h, const float* map, const float* fluid, const OracleOptions* o, int n,
                   const double* nx, const double* ny, const double* time, double* rgb, OracleEnd* ends);

/* A whole frame into hdr (width * height * 4 floats: RGB and the pixel-class bits), rows [y0, y1).
 * jitter 0: the reference's stratified side x side samples (lens.inc:365-377); n > 0: n rays a pixel at
 * the seeded offsets of oracleJitter.  threads: 0 all cores.  ends: width*height*rays records or NULL. */
void oracleRender32(const OracleFrame* h, const float* map, const float* fluid, const OracleOptions* o, int jitter,
                    uint32_t seed, int threads, int y0, int y1, float* hdr, OracleEnd* ends);
void oracleRender64(const OracleFrame* h32, const OracleFrame64* h, const float* map, const float* fluid,
                    const OracleOptions* o, int jitter, uint32_t seed, int threads, int y0, int y1, double* hdr,
                    OracleEnd* ends);

/* The sub-pixel offset of ray k of a pixel (jittered sampling): two uniform values in [0, 1) with 24
 * bits, from a hash of (seed, pixel index, k). */
void oracleJitter(uint32_t seed, uint32_t pixel, uint32_t k, float* dx, float* dy);

/* The bloom pyramid and tone map of a frame's light (width * height * 4 floats) to BGRA (postOracle.c). */
void oraclePost(const OracleFrame* h, const float* hdr, uint32_t* bgra);

/* The disc fluid (fluidOracle.c, after src/scene/fluid.c): made for a disc and a moment, advanced to a
 * later moment in steps of 0.2 (returns whether it stepped), its field (1024 x 256 floats) and moment. */
typedef struct OracleFluid OracleFluid;
OracleFluid* oracleFluidNew(float inner, float outer, float spin, double time);
int oracleFluidAdvance(OracleFluid* f, double time);
double oracleFluidRead(const OracleFluid* f, float* out);
void oracleFluidFree(OracleFluid* f);

/* The reference's painted disc (discOracle.c, after hole.c:136-178 buildDisc): gas, dust, colours and
 * sky into a whole map (ring tables left as they are); and the ring tables for a disc (hole.c:186). */
void oraclePaintDisc(float* map);
/* The unscaled gas's inner-half sum in texel order and in the GPU painter's order (`blocks` runs), and
 * the float scale each gives (sums[2], scales[2]). */
void oracleGasSums(int blocks, double* sums, float* scales);
void oracleSetRings(float* map, float inner, float outer, float spin);

#endif
