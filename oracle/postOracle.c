/* The oracle's bloom pyramid and tone map (test infrastructure, see oracle.h): the software backend's
 * bloomTap / bloomDownRow / bloomUpRow (eugeniobenfica/artful v0.4.0 src/software/software.c:320-387)
 * and lensToneMap / lensFill (src/software/lens.inc:387-440), one pixel at a time, with the same float
 * operations in the same order (built with -ffp-contract=off).  Pinned bit for bit against the
 * reference's own renderer (tests/golden/, oracle/refHarness.c refDraw). */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static float minRef(float a, float b) { return b < a ? b : a; }   /* core.h:64 artfMinf */
static float maxRef(float a, float b) { return a < b ? b : a; }   /* core.h:65 artfMaxf */
static int clampRef(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }
static float minLane(float a, float b) { return a < b ? a : b; }  /* simd.h:230 v8fMin */
static float maxLane(float a, float b) { return a > b ? a : b; }  /* simd.h:231 v8fMax */

static float bright(float v) { return minRef(maxRef(v - 2.f, 0.f), 48.f); }

/* software.c:320-328 */
static float tapAt(const float* level, int width, int height, float sx, float sy) {
    const float baseX = floorf(sx), baseY = floorf(sy), partX = sx - baseX, partY = sy - baseY;
    const int x0 = clampRef((int)baseX, 0, width - 1), x1 = clampRef((int)baseX + 1, 0, width - 1);
    const float* r0 = level + (size_t)clampRef((int)baseY, 0, height - 1) * width;
    const float* r1 = level + (size_t)clampRef((int)baseY + 1, 0, height - 1) * width;
    const float top = r0[x0] + (r0[x1] - r0[x0]) * partX, bottom = r1[x0] + (r1[x1] - r1[x0]) * partX;
    return top + (bottom - top) * partY;
}

static uint32_t ditherHash(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t h = x * 73856093u ^ y * 19349663u ^ z * 83492791u;
    h = (h ^ h >> 15) * 0x2C1B3C6Du;
    h = (h ^ h >> 12) * 0x297A2D39u;
    return h ^ h >> 15;
}

static float toneCurve(float x) {
    const float top = x * (x * 2.51f + .03f);
    const float bottom = x * (x * 2.43f + .59f) + .14f;
    return sqrtf(minLane(top / bottom, 1.f));
}

/* hdr: width * height * 4 floats (RGB and a fourth value, ignored); bgra: width * height. */
void oraclePost(const OracleFrame* h, const float* hdr, uint32_t* bgra) {
    const int width = (int)h->size[0], height = (int)h->size[1], levels = (int)h->size[3];
    size_t bloomPixels = 0;
    for (int i = 0; i < levels; ++i) bloomPixels += (size_t)h->bloom[i][1] * h->bloom[i][2];
    float* planes = (float*)calloc(bloomPixels * 3 + 1, sizeof(float));
    if (!planes) return;
    float* bloom[3] = {planes, planes + bloomPixels, planes + 2 * bloomPixels};
    /* software.c:333-365: down */
    for (int L = 0; L < levels; ++L) {
        const uint32_t* to = h->bloom[L];
        for (uint32_t y = 0; y < to[2]; ++y)
            for (int c = 0; c < 3; ++c) {
                float* out = bloom[c] + to[0] + (size_t)y * to[1];
                if (L == 0) {
                    const int lastX = width - 1, lastY = height - 1;
                    const int y0 = (int)y * 2 < lastY ? (int)y * 2 : lastY, y1 = (int)y * 2 + 1 < lastY ? (int)y * 2 + 1 : lastY;
                    for (uint32_t x = 0; x < to[1]; ++x) {
                        const int x0 = (int)x * 2 < lastX ? (int)x * 2 : lastX, x1 = (int)x * 2 + 1 < lastX ? (int)x * 2 + 1 : lastX;
                        const float* a = hdr + (size_t)y0 * width * 4;
                        const float* b = hdr + (size_t)y1 * width * 4;
                        out[x] = (bright(a[x0 * 4 + c]) + bright(a[x1 * 4 + c]) + bright(b[x0 * 4 + c]) +
                                  bright(b[x1 * 4 + c])) * .25f;
                    }
                } else {
                    const uint32_t* from = h->bloom[L - 1];
                    const float cy = (float)y * 2.f + .5f;
                    for (uint32_t x = 0; x < to[1]; ++x) {
                        const float cx = (float)x * 2.f + .5f;
                        float sum = 0;
                        for (int k = 0; k < 4; ++k)
                            sum += tapAt(bloom[c] + from[0], (int)from[1], (int)from[2], cx + (k & 1 ? 1.f : -1.f),
                                         cy + (k & 2 ? 1.f : -1.f));
                        out[x] = sum * .25f;
                    }
                }
            }
    }
    /* software.c:368-386: up, from the top */
    for (int L = levels - 1; L-- > 0;) {
        const uint32_t* to = h->bloom[L];
        const uint32_t* from = h->bloom[L + 1];
        for (uint32_t y = 0; y < to[2]; ++y) {
            const float sy = ((float)y + .5f) * .5f - .5f;
            for (int c = 0; c < 3; ++c) {
                float* out = bloom[c] + to[0] + (size_t)y * to[1];
                for (uint32_t x = 0; x < to[1]; ++x) {
                    const float sx = ((float)x + .5f) * .5f - .5f;
                    float sum = 0;
                    for (int k = 0; k < 4; ++k)
                        sum += tapAt(bloom[c] + from[0], (int)from[1], (int)from[2], sx + (k & 1 ? .5f : -.5f),
                                     sy + (k & 2 ? .5f : -.5f));
                    out[x] += sum * (.25f * .85f);
                }
            }
        }
    }
    /* lens.inc:395-440 */
    const float exposure = h->image[0], spread = h->look[3] * (1.f - .85f);
    const uint32_t* level = h->bloom[0];
    const int bw = (int)level[1], bh = (int)level[2];
    for (int y = 0; y < height; ++y) {
        const float sy = ((float)y + .5f) * .5f - .5f, baseY = floorf(sy), partY = sy - baseY;
        const int y0 = clampRef((int)baseY, 0, bh - 1), y1 = clampRef((int)baseY + 1, 0, bh - 1);
        for (int x = 0; x < width; ++x) {
            const float sx = ((float)x + .5f) * .5f - .5f;
            const float baseX = floorf(sx), partX = sx - baseX;
            const int x0 = (int)minLane(maxLane(baseX, 0.f), (float)(bw - 1));
            const int x1 = (int)minLane(maxLane(baseX + 1.f, 0.f), (float)(bw - 1));
            float glows[3];
            for (int c = 0; c < 3; ++c) {
                const float* plane = bloom[c] + level[0];
                const float a = plane[y0 * bw + x0], b = plane[y0 * bw + x1];
                const float d = plane[y1 * bw + x0], e = plane[y1 * bw + x1];
                const float upper = a + (b - a) * partX, lower = d + (e - d) * partX;
                glows[c] = upper + (lower - upper) * partY;
            }
            const float grey = glows[0] * .3f + glows[1] * .59f + glows[2] * .11f;
            const float dither = (float)(int)(ditherHash((uint32_t)(x + y * 8192), 7u, 13u) & 255u) * (1.f / 255.f);
            uint32_t bytes[3];
            for (int c = 0; c < 3; ++c) {
                const float glow = glows[c] + (grey - glows[c]) * .9f;
                const float light = hdr[((size_t)y * width + x) * 4 + c] + glow * spread;
                bytes[c] = (uint32_t)(int)minLane(toneCurve(light * exposure) * 255.f + dither, 255.f);
            }
            bgra[(size_t)y * width + x] = bytes[0] << 16 | bytes[1] << 8 | bytes[2] | 0xFF000000u;
        }
    }
    free(planes);
}
