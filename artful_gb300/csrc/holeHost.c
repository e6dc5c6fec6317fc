/* artful_cuda — the host side of the hole, in C11: what every frame's trace reads and that is the
 * same for all of its rays.  A restatement of the reference's src/scene/hole.c for this path:
 *
 *   artfCudaBlackHoleDefaults  hole.c:225-240   artfCudaIsco       hole.c:199-213
 *   artfCudaHoleClamp          hole.c:245-258   artfCudaOrbitSpeed hole.c:215-223
 *   artfCudaHoleFrame          hole.c:273-371
 *
 * and the gas's clock (fluid.c:319-333), the FP64 frame and the scenes of the five physical parameters.
 * The ring and colour tables and the synthetic scenes are in synthScene.c.  The FP32 frame keeps the
 * reference's order of operations, with no contraction (this file is built with -ffp-contract=off),
 * because the FP32 trace is checked bit for bit against the reference's. */
#include "artful_cuda.h"

#include <math.h>
#include <string.h>

typedef ArtfCudaVec3 Vec;

static Vec vec(float x, float y, float z) { Vec v = {x, y, z}; return v; }
static Vec vsub(Vec a, Vec b) { return vec(a.x - b.x, a.y - b.y, a.z - b.z); }
static Vec vscale(Vec a, float s) { return vec(a.x * s, a.y * s, a.z * s); }
static float vdot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static Vec vcross(Vec a, Vec b) { return vec(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static float vlength(Vec a) { return sqrtf(vdot(a, a)); }
static Vec vnormalize(Vec a) {
    const float l = vlength(a);
    return l > 0 ? vscale(a, 1.f / l) : a;
}
/* (the reference's artfMinf / artfMaxf / artfClampf: which operand wins a tie or a NaN matters for bits) */
static float fminRef(float a, float b) { return b < a ? b : a; }
static float fmaxRef(float a, float b) { return a < b ? b : a; }
static float fclampRef(float v, float lo, float hi) { return v < lo ? lo : v > hi ? hi : v; }

/* ---- orbits ------------------------------------------------------------------------------------- */

/* x^(1/3) for x > 0 by Newton's iteration, 60 rounds from max(x, 1): converged to the last bit. */
static double cubeRootNewton(double x) {
    if (x <= 0) return 0;
    double v = x > 1 ? x : 1;
    for (int i = 0; i < 60; ++i) v = (2.0 * v + x / (v * v)) / 3.0;
    return v;
}

/* Bardeen, Press & Teukolsky (1972): the ISCO radius of a Kerr hole, prograde for spin > 0. */
float artfCudaIsco(float spin) {
    const double a = spin, a2 = a * a;
    const double z1 = 1.0 + cubeRootNewton(1.0 - a2) * (cubeRootNewton(1.0 + a) + cubeRootNewton(1.0 - a));
    const double z2 = sqrt(3.0 * a2 + z1 * z1);
    const double root = sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2));
    return (float)(3.0 + z2 - (a < 0 ? -root : root));
}

/* A circular equatorial orbit's speed, measured by the zero-angular-momentum observer there. */
float artfCudaOrbitSpeed(float spin, float r) {
    const double a = spin, rr = (double)r * r, delta = rr - 2.0 * r + a * a;
    const double big = (rr + a * a) * (rr + a * a) - a * a * delta;
    const double omega = 1.0 / ((double)r * sqrt((double)r) + a), frameDrag = 2.0 * a * r / big;
    const double varpi = sqrt(big) / r, lapse = r * sqrt(delta) / sqrt(big);
    const double v = (omega - frameDrag) * varpi / lapse;
    return (float)(v > .99 ? .99 : v);
}

/* ---- the description ------------------------------------------------------------------------------ */

ArtfCudaBlackHoleDesc artfCudaBlackHoleDefaults(void) {
    ArtfCudaBlackHoleDesc d;
    memset(&d, 0, sizeof d);
    d.axis = vec(0, -1, 0);
    d.mass = 1.f;
    d.spin = .6f;
    d.discOuter = 34.f;
    d.discHeight = .03f;
    d.discThickness = 1.f;
    d.discGain = 2.1f;
    d.stars = .4f;
    d.bloom = 4.5f;
    d.exposure = 1.f;
    d.samples = 1;
    return d;
}

void artfCudaHoleClamp(const ArtfCudaBlackHoleDesc* in, ArtfCudaBlackHoleDesc* out) {
    ArtfCudaBlackHoleDesc d = *in;
    const float spin = fclampRef(in->spin, -.998f, .998f);
    const float horizon = 1.f + sqrtf(1.f - spin * spin);
    const float inner = in->discInner > 0 ? fmaxRef(in->discInner, horizon + .2f) : artfCudaIsco(spin);
    d.spin = spin;
    d.mass = fmaxRef(in->mass, 1e-6f);
    d.discInner = inner;
    d.discOuter = fmaxRef(in->discOuter, inner + 1.f);
    d.discHeight = fmaxRef(in->discHeight, 1e-3f);
    d.samples = in->samples < 1 ? 1 : in->samples > 8 ? 8 : in->samples;
    *out = d;
}

/* ---- the frame ---------------------------------------------------------------------------------- */

/* The disc's frame (x, y = axis, z) for a hole axis: its own basis, so that the disc lies in xz. */
typedef struct DiscBasis { Vec ex, ey, ez; } DiscBasis;

static DiscBasis discBasis(Vec axis) {
    DiscBasis b;
    const Vec given = vlength(axis) > 0 ? vnormalize(axis) : vec(0, 1, 0);
    const Vec other = fabsf(given.z) < .9f ? vec(0, 0, 1) : vec(1, 0, 0);
    b.ex = vnormalize(vcross(given, other));
    b.ey = given;
    b.ez = vcross(b.ex, b.ey);
    return b;
}

/* A world vector in the eye's (r, theta, phi) directions: first into the disc frame in the trace's
 * order (x, z, axis), then onto the three directions. */
static void toLocal(Vec v, const DiscBasis* b, Vec er, Vec etheta, Vec ephi, float w, float* o) {
    const Vec h = vec(vdot(v, b->ex), vdot(v, b->ez), vdot(v, b->ey));
    o[0] = vdot(h, er);
    o[1] = vdot(h, etheta);
    o[2] = vdot(h, ephi);
    o[3] = w;
}

static uint32_t bloomLevels(int width, int height, uint32_t (*bloom)[4], uint32_t* levelsOut) {
    uint32_t w = (uint32_t)width, h = (uint32_t)height, at = 0, levels = 0;
    while (levels < ARTF_CUDA_BLOOM_LEVELS && (!levels || (w > 3 && h > 3))) {
        w = (w + 1) / 2;
        h = (h + 1) / 2;
        bloom[levels][0] = at;
        bloom[levels][1] = w;
        bloom[levels][2] = h;
        at += w * h;
        ++levels;
    }
    *levelsOut = levels;
    return at;
}

uint32_t artfCudaHoleFrame(const ArtfCudaCamera* c, const ArtfCudaBlackHoleDesc* d, double fluidTime, int width,
                           int height, ArtfCudaHoleFrame* out) {
    if (!c || !d || !out || width < 1 || height < 1) return 0;
    memset(out, 0, sizeof *out);
    const float a = d->spin, horizon = 1.f + sqrtf(1.f - a * a);
    const DiscBasis b = discBasis(d->axis);

    /* the eye in masses, kept at least 0.3 above the horizon */
    Vec eye = vscale(vsub(c->position, d->position), 1.f / d->mass);
    float r = vlength(eye);
    const float least = horizon + .3f;
    if (r < least) {
        eye = r > 0 ? vscale(eye, least / r) : vec(0, 0, least);
        r = least;
    }
    const float px = vdot(eye, b.ex) / r, py = vdot(eye, b.ey) / r, pz = vdot(eye, b.ez) / r;
    const float sine = sqrtf(px * px + pz * pz);
    const float cx = sine > 1e-5f ? px / sine : 1.f, cz = sine > 1e-5f ? pz / sine : 0.f;
    const Vec er = vec(px, pz, py), etheta = vec(py * cx, py * cz, -sine), ephi = vec(-cz, cx, 0);
    out->er[0] = er.x, out->er[1] = er.y, out->er[2] = er.z, out->er[3] = r;
    out->etheta[0] = etheta.x, out->etheta[1] = etheta.y, out->etheta[2] = etheta.z;
    out->ephi[0] = ephi.x, out->ephi[1] = ephi.y, out->ephi[2] = ephi.z;

    /* Kerr's metric at the eye, in Boyer-Lindquist form, for the observer at rest in the dragged frame */
    const float mu = py, r2 = r * r, a2 = a * a;
    const float sigma = r2 + a2 * mu * mu, delta = r2 - 2.f * r + a2;
    const float big = (r2 + a2) * (r2 + a2) - a2 * delta * sine * sine;
    const float rho = sqrtf(sigma), rootDelta = sqrtf(delta), rootBig = sqrtf(big);
    const float varpiAxis = rootBig / rho;
    out->metric[0] = rho * rootDelta / rootBig;
    out->metric[1] = 2.f * a * r / big * varpiAxis * sine;
    out->metric[2] = varpiAxis * sine;
    out->metric[3] = varpiAxis;
    out->place[0] = rho;
    out->place[1] = rootDelta;
    out->place[2] = 1.f / r;
    out->place[3] = mu;
    out->spin[0] = a;
    out->spin[1] = .995f / horizon;
    out->spin[2] = d->discHeight;
    out->spin[3] = d->shutter;
    out->flow[0] = (float)fluidTime;

    /* the camera basis, scaled to the image's half extents, and the eye's velocity */
    const Vec forward = vnormalize(vsub(c->target, c->position));
    const Vec right = vnormalize(vcross(forward, c->up));
    const Vec up = vcross(right, forward);
    const float tanY = tanf(c->fovY * .5f), tanX = tanY * (float)width / (float)(height > 1 ? height : 1);
    toLocal(vscale(right, tanX), &b, er, etheta, ephi, 0.f, out->right);
    toLocal(vscale(up, tanY), &b, er, etheta, ephi, 0.f, out->up);
    toLocal(forward, &b, er, etheta, ephi, 0.f, out->forward);
    float speed = vlength(d->velocity);
    const Vec velocity = speed > .99f ? vscale(d->velocity, .99f / speed) : d->velocity;
    speed = fminRef(speed, .99f);
    toLocal(velocity, &b, er, etheta, ephi, 1.f / sqrtf(1.f - speed * speed), out->boost);

    out->disc[0] = d->discInner;
    out->disc[1] = d->discOuter;
    out->disc[2] = d->time;
    out->disc[3] = d->discThickness;
    out->look[0] = d->discGain;
    out->look[1] = d->doppler;
    out->look[2] = d->stars;
    out->look[3] = d->bloom;
    out->image[0] = d->exposure;
    out->image[1] = 2.f / (float)width;
    out->image[2] = 2.f / (float)height;
    out->image[3] = 1.f / (float)(d->samples * d->samples);
    out->size[0] = (uint32_t)width;
    out->size[1] = (uint32_t)height;
    out->size[2] = (uint32_t)d->samples;
    return bloomLevels(width, height, out->bloom, &out->size[3]);
}

/* ---- the frame in double ---------------------------------------------------------------------- */

typedef struct DVec { double x, y, z; } DVec;
static DVec dvec(double x, double y, double z) { DVec v = {x, y, z}; return v; }
static DVec dfrom(Vec v) { return dvec(v.x, v.y, v.z); }
static DVec dsub(DVec a, DVec b) { return dvec(a.x - b.x, a.y - b.y, a.z - b.z); }
static DVec dscale(DVec a, double s) { return dvec(a.x * s, a.y * s, a.z * s); }
static double ddot(DVec a, DVec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static DVec dcross(DVec a, DVec b) { return dvec(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static double dlength(DVec a) { return sqrt(ddot(a, a)); }
static DVec dnormalize(DVec a) {
    const double l = dlength(a);
    return l > 0 ? dscale(a, 1.0 / l) : a;
}

static void toLocal64(DVec v, const DVec* basis, DVec er, DVec etheta, DVec ephi, double w, double* o) {
    const DVec h = dvec(ddot(v, basis[0]), ddot(v, basis[2]), ddot(v, basis[1]));
    o[0] = ddot(h, er);
    o[1] = ddot(h, etheta);
    o[2] = ddot(h, ephi);
    o[3] = w;
}

/* A camera and a hole in double: what the FP64 frame is made from. */
typedef struct DScene {
    DVec position, target, up, holePosition, axis, velocity;
    double fovY, mass, spin, inner, outer, height, shutter, time, thickness, gain, doppler, stars, bloom, exposure;
    int samples;
} DScene;

static void frame64Of(const DScene* s, double fluidTime, int width, int height, ArtfCudaHoleFrame64* out) {
    memset(out, 0, sizeof *out);
    const double a = s->spin, horizon = 1.0 + sqrt(1.0 - a * a);
    DVec basis[3];
    {
        const DVec given = dlength(s->axis) > 0 ? dnormalize(s->axis) : dvec(0, 1, 0);
        const DVec other = fabs(given.z) < .9 ? dvec(0, 0, 1) : dvec(1, 0, 0);
        basis[0] = dnormalize(dcross(given, other));
        basis[1] = given;
        basis[2] = dcross(basis[0], basis[1]);
    }
    DVec eye = dscale(dsub(s->position, s->holePosition), 1.0 / s->mass);
    double r = dlength(eye);
    const double least = horizon + .3;
    if (r < least) {
        eye = r > 0 ? dscale(eye, least / r) : dvec(0, 0, least);
        r = least;
    }
    const double px = ddot(eye, basis[0]) / r, py = ddot(eye, basis[1]) / r, pz = ddot(eye, basis[2]) / r;
    const double sine = sqrt(px * px + pz * pz);
    const double cx = sine > 1e-5 ? px / sine : 1.0, cz = sine > 1e-5 ? pz / sine : 0.0;
    const DVec er = dvec(px, pz, py), etheta = dvec(py * cx, py * cz, -sine), ephi = dvec(-cz, cx, 0);
    out->er[0] = er.x, out->er[1] = er.y, out->er[2] = er.z, out->er[3] = r;
    out->etheta[0] = etheta.x, out->etheta[1] = etheta.y, out->etheta[2] = etheta.z;
    out->ephi[0] = ephi.x, out->ephi[1] = ephi.y, out->ephi[2] = ephi.z;
    const double mu = py, r2 = r * r, a2 = a * a;
    const double sigma = r2 + a2 * mu * mu, delta = r2 - 2.0 * r + a2;
    const double big = (r2 + a2) * (r2 + a2) - a2 * delta * sine * sine;
    const double rho = sqrt(sigma), rootDelta = sqrt(delta), rootBig = sqrt(big);
    const double varpiAxis = rootBig / rho;
    out->metric[0] = rho * rootDelta / rootBig;
    out->metric[1] = 2.0 * a * r / big * varpiAxis * sine;
    out->metric[2] = varpiAxis * sine;
    out->metric[3] = varpiAxis;
    out->place[0] = rho;
    out->place[1] = rootDelta;
    out->place[2] = 1.0 / r;
    out->place[3] = mu;
    out->spin[0] = a;
    out->spin[1] = .995 / horizon;
    out->spin[2] = s->height;
    out->spin[3] = s->shutter;
    out->flow[0] = fluidTime;
    const DVec forward = dnormalize(dsub(s->target, s->position));
    const DVec right = dnormalize(dcross(forward, s->up));
    const DVec up = dcross(right, forward);
    const double tanY = tan(s->fovY * .5), tanX = tanY * (double)width / (double)(height > 1 ? height : 1);
    toLocal64(dscale(right, tanX), basis, er, etheta, ephi, 0, out->right);
    toLocal64(dscale(up, tanY), basis, er, etheta, ephi, 0, out->up);
    toLocal64(forward, basis, er, etheta, ephi, 0, out->forward);
    DVec velocity = s->velocity;
    double speed = dlength(velocity);
    if (speed > .99) velocity = dscale(velocity, .99 / speed);
    if (speed > .99) speed = .99;
    toLocal64(velocity, basis, er, etheta, ephi, 1.0 / sqrt(1.0 - speed * speed), out->boost);
    out->disc[0] = s->inner;
    out->disc[1] = s->outer;
    out->disc[2] = s->time;
    out->disc[3] = s->thickness;
    out->look[0] = s->gain;
    out->look[1] = s->doppler;
    out->look[2] = s->stars;
    out->look[3] = s->bloom;
    out->image[0] = s->exposure;
    out->image[1] = 2.0 / width;
    out->image[2] = 2.0 / height;
    out->image[3] = 1.0 / ((double)s->samples * s->samples);
}

int artfCudaHoleFrame64(const ArtfCudaCamera* c, const ArtfCudaBlackHoleDesc* d, double fluidTime, int width,
                        int height, ArtfCudaHoleFrame64* out) {
    if (!c || !d || !out || width < 1 || height < 1) return ARTF_CUDA_EINVAL;
    DScene s;
    s.position = dfrom(c->position), s.target = dfrom(c->target), s.up = dfrom(c->up), s.fovY = c->fovY;
    s.holePosition = dfrom(d->position), s.axis = dfrom(d->axis), s.velocity = dfrom(d->velocity);
    s.mass = d->mass, s.spin = d->spin, s.inner = d->discInner, s.outer = d->discOuter, s.height = d->discHeight;
    s.shutter = d->shutter, s.time = d->time, s.thickness = d->discThickness, s.gain = d->discGain;
    s.doppler = d->doppler, s.stars = d->stars, s.bloom = d->bloom, s.exposure = d->exposure, s.samples = d->samples;
    frame64Of(&s, fluidTime, width, height, out);
    return ARTF_CUDA_OK;
}


/* ---- the gas's clock (src/scene/fluid.c:319-333, and its step's f->time += STEP at fluid.c:240) ------ */

#define FLUID_STEP .2f     /* a step's time, in float as the reference's STEP */
#define FLUID_MOST_STEPS 48

int artfCudaFluidClock(double* clock, double time) {
    if (!clock || !isfinite(time)) return 0;
    if (time - *clock < FLUID_STEP) {
        /* behind: no step; a clock set more than 8 back restarts the gas's clock there */
        if (time < *clock - 8.0) *clock = time;
        return 0;
    }
    /* (the gap in steps is capped before it becomes an int: a clock far ahead would overflow one) */
    const double gap = (time - *clock) / FLUID_STEP;
    int steps = gap >= (double)(FLUID_MOST_STEPS + 1) ? FLUID_MOST_STEPS + 1 : (int)gap;
    if (steps > FLUID_MOST_STEPS) {
        *clock = time - (double)FLUID_MOST_STEPS * FLUID_STEP;
        steps = FLUID_MOST_STEPS;
    }
    for (int i = 0; i < steps; ++i) *clock += FLUID_STEP;
    return steps;
}


/* ---- scenes by their five physical parameters (the adjoint's) ------------------------------------ */

/* The ISCO in double (the same formula as artfCudaIsco, without its rounding to float). */
static double iscoDouble(double a) {
    const double a2 = a * a;
    const double z1 = 1.0 + cubeRootNewton(1.0 - a2) * (cubeRootNewton(1.0 + a) + cubeRootNewton(1.0 - a));
    const double z2 = sqrt(3.0 * a2 + z1 * z1);
    const double root = sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2));
    return 3.0 + z2 - (a < 0 ? -root : root);
}

static DScene paramsScene(const ArtfCudaHoleParams* p, const double* theta) {
    DScene s;
    memset(&s, 0, sizeof s);
    const double a = theta[0], i = theta[1], scale = theta[2], r = theta[4];
    s.position = dvec(0.0, r * cos(i), r * sin(i));
    s.target = dvec(0, 0, 0);
    s.up = dvec(0, 1, 0);
    s.fovY = p->fovY;
    s.holePosition = dvec(0, 0, 0);
    s.axis = dvec(0, 1, 0);
    s.velocity = dvec(0, 0, 0);
    s.mass = 1.0, s.spin = a, s.inner = scale * iscoDouble(a), s.outer = p->outer, s.height = p->height;
    s.shutter = 0.0, s.time = p->time, s.thickness = p->thickness, s.gain = p->gain, s.doppler = p->doppler;
    s.stars = p->stars, s.bloom = 0.0, s.exposure = 1.0, s.samples = 1;
    return s;
}

static void thetaOf(const ArtfCudaHoleParams* p, double* theta) {
    theta[0] = p->spin, theta[1] = p->inclination, theta[2] = p->innerScale, theta[3] = p->emissivity;
    theta[4] = p->distance;
}

/* The scenes the parameters may name: the reference's spin range (|a| <= 0.998), an eye outside the
 * clamp radius at any inclination, a disc whose inner edge lies inside its outer edge, finite values,
 * and a margin of the differencing step on every bound. */
static int paramsValid(const ArtfCudaHoleParams* p) {
    const double v[] = {p->spin, p->inclination, p->innerScale, p->emissivity, p->distance, p->fovY, p->outer,
                        p->height, p->thickness, p->gain, p->doppler, p->stars, p->time};
    for (size_t k = 0; k < sizeof v / sizeof v[0]; ++k)
        if (!isfinite(v[k])) return 0;
    if (!(fabs(p->spin) <= .998) || !(p->inclination >= 0.0 && p->inclination <= 3.141592653589793)) return 0;
    if (!(p->innerScale > 0.0) || !(p->distance >= 4.0) || !(p->fovY > 0.0 && p->fovY < 3.1)) return 0;
    if (!(p->height > 0.0) || !(p->thickness >= 0.0) || !(p->stars >= 0.0)) return 0;
    return p->outer > p->innerScale * iscoDouble(p->spin) * 1.001;
}

int artfCudaHoleParamsScene(const ArtfCudaHoleParams* p, ArtfCudaCamera* camera, ArtfCudaBlackHoleDesc* desc) {
    if (!p || !camera || !desc || !paramsValid(p)) return ARTF_CUDA_EINVAL;
    double theta[5];
    thetaOf(p, theta);
    const DScene s = paramsScene(p, theta);
    memset(camera, 0, sizeof *camera);
    camera->position = vec((float)s.position.x, (float)s.position.y, (float)s.position.z);
    camera->up = vec(0, 1, 0);
    camera->fovY = (float)p->fovY;
    camera->near_ = .1f;
    *desc = artfCudaBlackHoleDefaults();
    desc->axis = vec(0, 1, 0);
    desc->spin = (float)s.spin;
    desc->discInner = (float)s.inner;
    desc->discOuter = (float)s.outer;
    desc->discHeight = (float)s.height;
    desc->discThickness = (float)s.thickness;
    desc->discGain = (float)s.gain;
    desc->doppler = (float)s.doppler;
    desc->stars = (float)s.stars;
    desc->bloom = 0.f;
    desc->exposure = 1.f;
    desc->time = (float)s.time;
    desc->samples = 1;
    return ARTF_CUDA_OK;
}

/* The frame fields the gradient flows through, in the order of ArtfCudaHoleParams' Jacobian rows. */
static void gradFields(const ArtfCudaHoleFrame64* f, double* out) {
    int k = 0;
    for (int c = 0; c < 3; ++c) out[k++] = f->forward[c];
    for (int c = 0; c < 3; ++c) out[k++] = f->right[c];
    for (int c = 0; c < 3; ++c) out[k++] = f->up[c];
    for (int c = 0; c < 4; ++c) out[k++] = f->metric[c];
    for (int c = 0; c < 4; ++c) out[k++] = f->place[c];
    for (int c = 0; c < 3; ++c) out[k++] = f->er[c];
    for (int c = 0; c < 3; ++c) out[k++] = f->etheta[c];
    for (int c = 0; c < 3; ++c) out[k++] = f->ephi[c];
    out[k++] = f->spin[0];
    out[k++] = f->disc[0];
}

int artfCudaHoleParamsFrames(const ArtfCudaHoleParams* p, int width, int height, ArtfCudaHoleFrame* f32,
                             ArtfCudaHoleFrame64* f64, double* jacobian) {
    if (!p || width < 1 || height < 1 || !paramsValid(p)) return ARTF_CUDA_EINVAL;
    double theta[5];
    thetaOf(p, theta);
    if (f32) {
        ArtfCudaCamera camera;
        ArtfCudaBlackHoleDesc desc;
        artfCudaHoleParamsScene(p, &camera, &desc);
        if (!artfCudaHoleFrame(&camera, &desc, desc.time, width, height, f32)) return ARTF_CUDA_EINVAL;
    }
    if (f64) {
        const DScene s = paramsScene(p, theta);
        frame64Of(&s, s.time, width, height, f64);
    }
    if (jacobian) {
        /* central differences of the double frame, step 1e-6 of each parameter's scale */
        for (int q = 0; q < 5; ++q) {
            double up[5], down[5];
            memcpy(up, theta, sizeof up);
            memcpy(down, theta, sizeof down);
            const double h = 1e-6 * (fabs(theta[q]) > 1.0 ? fabs(theta[q]) : 1.0);
            up[q] += h;
            down[q] -= h;
            ArtfCudaHoleFrame64 fu, fd;
            const DScene su = paramsScene(p, up), sd = paramsScene(p, down);
            frame64Of(&su, su.time, width, height, &fu);
            frame64Of(&sd, sd.time, width, height, &fd);
            double gu[ARTF_CUDA_GRAD_FIELDS], gd[ARTF_CUDA_GRAD_FIELDS];
            gradFields(&fu, gu);
            gradFields(&fd, gd);
            for (int k = 0; k < ARTF_CUDA_GRAD_FIELDS; ++k) jacobian[k * 5 + q] = (gu[k] - gd[k]) / (2.0 * h);
        }
    }
    return ARTF_CUDA_OK;
}

int artfCudaHoleParamsMap(const ArtfCudaHoleParams* p, float* map) {
    if (!p || !map) return ARTF_CUDA_EINVAL;
    ArtfCudaCamera camera;
    ArtfCudaBlackHoleDesc desc;
    artfCudaHoleParamsScene(p, &camera, &desc);
    const ArtfCudaSynthDesc synth = {p->seed, desc.discInner, desc.discOuter, desc.spin, (float)p->emissivity, 2000};
    return artfCudaSynthMap(&synth, map);
}
