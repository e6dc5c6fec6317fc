/* The oracle's per-ray trace, written once for a scalar type REAL and included twice by lensOracle.c
 * (REAL float, then double).  Every line cites the reference statement it restates
 * (src/software/lens.inc of eugeniobenfica/artful v0.4.0); within each expression the operations
 * are in the reference's order, because in float that order decides the bits.
 *
 * Expects: REAL, FRAME (the frame struct), SFX (a name suffix), SQRT, FLOOR, FABS. */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)
#define K(v) ((REAL)(v##f)) /* the reference's float constants, in REAL */

/* x86's min and max (simd.h:1-5, 230-231): with a NaN, the second operand. */
static inline REAL FN(minX)(REAL a, REAL b) { return a < b ? a : b; }
static inline REAL FN(maxX)(REAL a, REAL b) { return a > b ? a : b; }
/* float -> int32 by truncation, as cvttps2dq (simd.h:185); NaN and out of range give INT32_MIN there */
static inline int32_t FN(toInt)(REAL x) {
    return (x > (REAL)-2147483648.0 && x < (REAL)2147483648.0) ? (int32_t)x : INT32_MIN;
}
/* a map read with the index kept in the map: the reference reads the same texels for every index
 * that is in range, and no case here reaches outside it */
static inline REAL FN(texel)(const float* base, int64_t i, int64_t count) {
    return (REAL)base[i < 0 ? 0 : i >= count ? count - 1 : i];
}

/* lens.inc:30-41 lensTurns: the angle of (x, y) in turns, by a polynomial arctangent. */
static REAL FN(turnsOf)(REAL y, REAL x) {
    const REAL ax = FABS(x), ay = FABS(y);
    const REAL most = FN(maxX)(FN(maxX)(ax, ay), K(1e-20)), least = FN(minX)(ax, ay);
    const REAL a = least / most, s = a * a;
    REAL r = K(-.0464964749) * s + K(.15931422);
    r = r * s - K(.327622764);
    r = r * s * a + a;
    if (ay > ax) r = K(1.57079633) - r;
    if (x < 0) r = K(3.14159265) - r;
    if (y < 0) r = 0 - r;
    return r * K(.15915494);
}

/* lens.inc:44-54 lensSine: the sine of an angle in turns. */
static REAL FN(sineOf)(REAL turns) {
    REAL t = turns - FLOOR(turns + K(.5));
    if (t > K(.25)) t = K(.5) - t;
    if (t < K(-.25)) t = K(-.5) - t;
    const REAL x = t * K(6.2831853), x2 = x * x;
    REAL p = x2 * K(2.7557319e-6) + K(-1.9841270e-4);
    p = p * x2 + K(8.3333333e-3);
    p = p * x2 + K(-.16666667);
    return p * x2 * x + x;
}

/* lens.inc:89-96 lensRow: a row of a region (starting `at` floats into a buffer of `count`) at a turn,
 * linear between two of its width (a power of two) columns. */
static REAL FN(rowAt)(const float* buffer, int64_t count, int64_t at, int width, int32_t row, REAL turn) {
    const REAL pos = (turn - FLOOR(turn)) * (REAL)width;
    const REAL column = FLOOR(pos), part = pos - column;
    const int32_t base = (int32_t)((uint32_t)row * (uint32_t)width);
    const int32_t c0 = FN(toInt)(column) & (width - 1), c1 = (c0 + 1) & (width - 1);
    const REAL a = FN(texel)(buffer, at + base + c0, count), b = FN(texel)(buffer, at + base + c1, count);
    return a + (b - a) * part;
}

/* lens.inc:69-86 lensStars: one layer of hashed-cube stars, added to rgb. */
static void FN(starLayer)(REAL dx_, REAL dy_, REAL dz_, REAL cells, int32_t density, REAL size, REAL gain, REAL* rgb) {
    const REAL px = dx_ * cells, py = dy_ * cells, pz = dz_ * cells;
    const REAL cx = FLOOR(px), cy = FLOOR(py), cz = FLOOR(pz);
    const uint32_t h = oracleCubeHash((uint32_t)FN(toInt)(cx), (uint32_t)FN(toInt)(cy), (uint32_t)FN(toInt)(cz));
    if (!(density > (int32_t)(h & 255))) return;
#define BYTE_OF(shift) ((REAL)(float)(int32_t)((h >> (shift)) & 255) * (REAL)(1.f / 255.f))
    const REAL ex = px - cx - BYTE_OF(8), ey = py - cy - BYTE_OF(16), ez = pz - cz - BYTE_OF(24);
    const REAL d2 = ex * ex + ey * ey + ez * ez;
    REAL light = FN(maxX)((REAL)1 - d2 * (REAL)(1.f / ((float)size * (float)size)), 0);
    light = light * light * gain;
    const REAL warm = BYTE_OF(3);
#undef BYTE_OF
    rgb[0] = rgb[0] + light * (K(.75) + warm * K(.25));
    rgb[1] = rgb[1] + light * K(.82);
    rgb[2] = rgb[2] + light * ((REAL)1 - warm * K(.45));
}

/* lens.inc:99-351 lensTrace for one ray. */
static void FN(traceRay)(const FRAME* h, const float* map, const float* fluid, REAL stepScale, REAL nx, REAL ny,
                         REAL time, REAL* out, OracleEnd* end) {
    const int64_t mapCount = ORACLE_MAP_FLOATS, fluidCount = ORACLE_FLUID_WIDTH * ORACLE_FLUID_HEIGHT;
    /* 101-107: the ray's direction at the eye, normalised */
    REAL dx = h->forward[0] + nx * h->right[0] + ny * h->up[0];
    REAL dy = h->forward[1] + nx * h->right[1] + ny * h->up[1];
    REAL dz = h->forward[2] + nx * h->right[2] + ny * h->up[2];
    const REAL invLength = (REAL)1 / SQRT(dx * dx + dy * dy + dz * dz);
    dx = dx * invLength, dy = dy * invLength, dz = dz * invLength;

    /* 110-122: aberration for a moving eye */
    REAL moved = 1;
    const REAL gamma = h->boost[3];
    if (gamma > 1) {
        const REAL bx = h->boost[0], by = h->boost[1], bz = h->boost[2], share = gamma / (gamma + 1);
        const REAL c = 0 - (dx * bx + dy * by + dz * bz);
        const REAL push = gamma * ((REAL)1 + share * c);
        const REAL over = (REAL)1 / (gamma * ((REAL)1 + c));
        dx = (dx - bx * push) * over;
        dy = (dy - by * push) * over;
        dz = (dz - bz * push) * over;
        moved = over;
    }

    /* 125-142: constants of motion and the equations' coefficients */
    const REAL a = h->spin[0], a2 = a * a, rho = h->place[0], rootDelta = h->place[1], u0 = h->place[2],
               mu0 = h->place[3];
    const REAL energy = h->metric[0] - h->metric[1] * dz;
    const REAL invEnergy = (REAL)1 / energy;
    const REAL xi = 0 - h->metric[2] * dz * invEnergy;
    const REAL xiAxis = h->metric[3] * dz * invEnergy;
    const REAL across = rho * dy * invEnergy;
    const REAL eta = across * across + mu0 * mu0 * (xiAxis * xiAxis - a2);
    const REAL big = eta + xi * xi;
    const REAL step = K(.13089969) * stepScale / SQRT(FN(maxX)(big, K(4.)));
    const REAL step2 = step * step;
    const REAL uA = a2 - big;
    const REAL xiOff = xi - a;
    const REAL uB = K(3.) * (eta + xiOff * xiOff);
    const REAL uC = (K(-2.) * a2) * eta;
    const REAL xiA = xi * a;
    const REAL twoA2 = K(2.) * a2;
#define BEND(x) ((x) * (uA + (x) * (uB + (x) * uC)))
#define DRAG(x) ((-a) * (x) * (K(2.) - xiA * (x)) / FN(maxX)((REAL)1 - ((x) + (x)) + a2 * (x) * (x), K(1e-3)))

    /* 146-152: the initial state */
    REAL u = u0, w = ((-u0) * u0 * rootDelta * rho) * dx * invEnergy;
    REAL n[3] = {h->er[0], h->er[1], h->er[2]};
    REAL v[3];
    for (int c = 0; c < 3; ++c) v[c] = across * h->etheta[c] + xiAxis * h->ephi[c];
    REAL psi = 0, drag = a != 0 ? DRAG(u) : 0;

    const REAL inner = h->disc[0], thickness = h->disc[3], gain = h->look[0], doppler = h->look[1],
               discHeight = h->spin[2];
    const REAL rhoScale = (REAL)1 / ((REAL)1 - inner / h->disc[1]);

    REAL sum[3] = {0, 0, 0}, through = 1, away[3] = {0, 0, 0}, awayPsi = 0;
    int sky = 0, lit = 0, crossings = 0, steps = 0, kind = ORACLE_CAP;
    REAL hitR = (REAL)NAN, hitPhi = (REAL)NAN, mino = 0;
    const REAL uHorizon = h->spin[1];
    const int maxSteps = stepScale < (REAL).75 ? 384 : 192;

    /* (loop-invariant: the reference recomputes them each step, with the same result) */
    const REAL half = step * K(.5), eighth = step2 * K(.125), halfSquare = step2 * K(.5),
               sixthSquare = step2 * (REAL)(1.f / 6.f), sixth = step * (REAL)(1.f / 6.f);
    for (int i = 0; i < maxSteps; ++i) {
        /* 165-192: one Nystrom step, three evaluations of u'' and n'' */
        const REAL k1 = BEND(u);
        const REAL c1 = big + twoA2 * (n[2] * n[2]);
        const REAL a1[3] = {0 - c1 * n[0], 0 - c1 * n[1], a2 * n[2] - c1 * n[2]};
        const REAL midU = u + half * w + eighth * k1;
        REAL midN[3], endN[3], a2s[3], a3[3], nextN[3], nextV[3];
        for (int c = 0; c < 3; ++c) midN[c] = n[c] + half * v[c] + eighth * a1[c];
        const REAL k2 = BEND(midU);
        const REAL c2 = big + twoA2 * (midN[2] * midN[2]);
        a2s[0] = 0 - c2 * midN[0], a2s[1] = 0 - c2 * midN[1], a2s[2] = a2 * midN[2] - c2 * midN[2];
        const REAL endU = u + step * w + halfSquare * k2;
        for (int c = 0; c < 3; ++c) endN[c] = n[c] + step * v[c] + halfSquare * a2s[c];
        const REAL k3 = BEND(endU);
        const REAL c3 = big + twoA2 * (endN[2] * endN[2]);
        a3[0] = 0 - c3 * endN[0], a3[1] = 0 - c3 * endN[1], a3[2] = a2 * endN[2] - c3 * endN[2];
        /* 181-185: NEXT_P is p + h q + h^2/6 (a + 2 b); NEXT_V is q + h/6 (a + c + 4 b) */
        const REAL nextU = u + step * w + sixthSquare * (k1 + (k2 + k2));
        const REAL nextW = w + sixth * (k1 + k3 + K(4.) * k2);
        for (int c = 0; c < 3; ++c) {
            nextN[c] = n[c] + step * v[c] + sixthSquare * (a1[c] + (a2s[c] + a2s[c]));
            nextV[c] = v[c] + sixth * (a1[c] + a3[c] + K(4.) * a2s[c]);
        }
        REAL nextDrag = 0, nextPsi = 0;
        if (a != 0) {
            nextDrag = DRAG(nextU);
            nextPsi = psi + sixth * (drag + nextDrag + K(4.) * DRAG(midU));
        }
        ++steps;

        /* 195-291: through the disc's plane? */
        if (n[2] * nextN[2] < 0) {
            const REAL part = n[2] / (n[2] - nextN[2]);
            const REAL hu = part * step, hh = hu * hu * K(.5);
            const REAL uc = u + hu * w + hh * k1;
            const REAL rhoCenter = ((REAL)1 - inner * uc) * rhoScale;
            if (rhoCenter > K(-.03) && rhoCenter < K(1.02)) {
                ++crossings;
                const REAL wc = w + hu * k1;
                const REAL cx = n[0] + hu * v[0] + hh * a1[0], cy = n[1] + hu * v[1] + hh * a1[1];
                const REAL vx = v[0] + hu * a1[0], vy = v[1] + hu * a1[1], vz = v[2] + hu * a1[2];
                const REAL psiC = psi + part * (nextPsi - psi);
                const REAL dragC = drag + part * (nextDrag - drag);
                const REAL turn = FN(turnsOf)(cy, cx) + psiC * K(.15915494);
                const REAL rate = ((cx * vy - cy * vx) / FN(maxX)(cx * cx + cy * cy, K(1e-6)) + dragC) * K(.15915494);
                const REAL slope = wc / uc;
                const REAL speed2 = vx * vx + vy * vy + (vz * vz + slope * slope);
                const REAL mu = FN(maxX)(FABS(vz) / SQRT(speed2), K(.02));
                const REAL slant = thickness / (REAL)3 / mu;
                const REAL reach = FN(minX)(discHeight / FN(maxX)(FABS(vz), K(1e-5)), step * K(1.5));

                /* 221-259: three slices through the disc's depth, front to back */
                REAL glow = 0, clear = through;
                for (int k = 0; k < 3; ++k) {
                    const REAL t = (REAL)(((float)k + .5f) * (2.f / 3.f) - 1.f);
                    const REAL ds = reach * t;
                    const REAL uk = uc + wc * ds;
                    const REAL rhoK = ((REAL)1 - inner * uk) * rhoScale;
                    const int inside = rhoK > 0 && rhoK < 1;
                    const REAL rowPos = (inside ? rhoK : 0) * (REAL)(ORACLE_MAP_HEIGHT - 1);
                    const REAL rowFloor = FN(minX)(FLOOR(rowPos), (REAL)(ORACLE_MAP_HEIGHT - 2));
                    const REAL rowPart = rowPos - rowFloor;
                    const int32_t row0 = FN(toInt)(rowFloor), row1 = row0 + 1;
                    const REAL speed0 = FN(texel)(map, ORACLE_ROWS_AT + (int64_t)row0 + row0, mapCount);
                    const REAL speed1 = FN(texel)(map, ORACLE_ROWS_AT + (int64_t)row1 + row1, mapCount);
                    const REAL turnK = turn + (inside ? rate * ds : 0);
                    const REAL d0 = FN(rowAt)(map, mapCount, 0, ORACLE_MAP_WIDTH, row0, turnK - speed0 * time);
                    const REAL d1 = FN(rowAt)(map, mapCount, 0, ORACLE_MAP_WIDTH, row1, turnK - speed1 * time);
                    REAL density = d0 + (d1 - d0) * rowPart;
                    /* 238-245: the fluid, each ring turned on since it was stepped */
                    const REAL fluidPos = (inside ? rhoK : 0) * (REAL)(ORACLE_FLUID_HEIGHT - 1);
                    const REAL fluidFloor = FN(minX)(FLOOR(fluidPos), (REAL)(ORACLE_FLUID_HEIGHT - 2));
                    const int32_t fluidRow = FN(toInt)(fluidFloor);
                    const REAL fluidTurn = turnK - speed0 * (REAL)(time - h->flow[0]);
                    const REAL g0 = FN(rowAt)(fluid, fluidCount, 0, ORACLE_FLUID_WIDTH, fluidRow, fluidTurn);
                    const REAL g1 = FN(rowAt)(fluid, fluidCount, 0, ORACLE_FLUID_WIDTH, fluidRow + 1, fluidTurn);
                    const REAL gas = g0 + (g1 - g0) * (fluidPos - fluidFloor);
                    density = density * ((REAL)(1.f - .1f) + K(.1) * gas);
                    /* 247-250: dust */
                    const REAL dustPos = (inside ? rhoK : 0) * (REAL)(ORACLE_DUST_HEIGHT - 1);
                    const int32_t dustRow = FN(toInt)(FN(minX)(FLOOR(dustPos), (REAL)(ORACLE_DUST_HEIGHT - 1)));
                    const REAL dusty = FN(rowAt)(map, mapCount, ORACLE_DUST_AT, ORACLE_DUST_WIDTH,
                                                 dustRow, turnK - speed0 * time);
                    const REAL litShare = (REAL)1 - K(.97) * dusty;
                    /* 252-258: height in the disc, opacity, emission */
                    const REAL height = t * (reach / discHeight);
                    const REAL level = FN(maxX)((REAL)1 - vz * vz * (height * height), 0);
                    density = inside ? density * level : 0;
                    const REAL depth = slant * density * ((REAL)1 + K(25.) * dusty);
                    const REAL alpha = depth / ((REAL)1 + depth);
                    glow = glow + clear * alpha * (density * litShare);
                    clear = clear * ((REAL)1 - alpha);
                }

                /* 262-279: the ring's heat and glow, and the Doppler and gravitational shift */
                const REAL rhoSafe = FN(minX)(FN(maxX)(rhoCenter, 0), 1);
                const int32_t rowIndex = FN(toInt)(rhoSafe * (REAL)(ORACLE_MAP_HEIGHT - 1));
                REAL heat = FN(texel)(map, ORACLE_ROWS_AT + 1 + (int64_t)rowIndex + rowIndex, mapCount);
                const REAL gives = FN(texel)(map, ORACLE_GLOW_AT + (int64_t)rowIndex, mapCount);
                REAL light = gain * glow * gives;
                if (doppler != 0) {
                    const REAL safeU = FN(maxX)(uc, K(1e-4));
                    const REAL root = safeU * SQRT(safeU);
                    const REAL lift = (REAL)1 + a * root;
                    const REAL spinRate = root / lift;
                    const REAL beneath = FN(maxX)((REAL)1 - K(3.) * safeU + (K(2.) * a) * root, K(1e-4));
                    const REAL shift = SQRT(beneath) * (invEnergy * moved) / (lift * ((REAL)1 - spinRate * xi));
                    const REAL g = (REAL)1 + doppler * (shift - (REAL)1);
                    const REAL g2 = g * g;
                    light = light * (g2 * g2);
                    heat = heat * g;
                }
                /* 281-289: a black body's colour at that heat */
                const REAL colorPos = FN(minX)(heat * (REAL)(ORACLE_COLORS / 2), (REAL)(ORACLE_COLORS - 1));
                const int32_t color = FN(toInt)(colorPos);
                const int64_t at = ORACLE_COLORS_AT + (int64_t)color + color + color;
                const REAL rgb[3] = {FN(texel)(map, at, mapCount), FN(texel)(map, at + 1, mapCount),
                                     FN(texel)(map, at + 2, mapCount)};
                for (int c = 0; c < 3; ++c) sum[c] = sum[c] + light * rgb[c];
                through = clear;
                if (light > 0 && !lit) {
                    lit = 1;
                    hitR = (REAL)1 / uc;
                    hitPhi = turn - FLOOR(turn);
                }
            }
        }

        /* 294-305: out, or in */
        if (0 > nextU) {
            const REAL part = u / (u - nextU);
            for (int c = 0; c < 3; ++c) away[c] = n[c] + part * (nextN[c] - n[c]);
            awayPsi = psi + part * (nextPsi - psi);
            sky = 1;
            kind = ORACLE_SKY;
            mino = ((REAL)i + part) * step;
            break;
        }
        if (nextU > uHorizon) { kind = ORACLE_HORIZON; mino = (REAL)(i + 1) * step; break; }
        if (!(through > K(.004))) { kind = ORACLE_OPAQUE; mino = (REAL)(i + 1) * step; break; }
        u = nextU;
        w = nextW;
        for (int c = 0; c < 3; ++c) n[c] = nextN[c], v[c] = nextV[c];
        psi = nextPsi;
        drag = nextDrag;
        if (i + 1 == maxSteps) mino = (REAL)maxSteps * step;
    }
#undef BEND
#undef DRAG

    /* 316-347: the sky behind, turned by the frame drag */
    REAL dir[3] = {0, 0, 0};
    if (sky) {
        const REAL invAway = (REAL)1 / SQRT(FN(maxX)(away[0] * away[0] + away[1] * away[1] + away[2] * away[2], K(1e-12)));
        const REAL psiTurns = awayPsi * K(.15915494);
        const REAL sine = FN(sineOf)(psiTurns), cosine = FN(sineOf)(psiTurns + K(.25));
        const REAL x = away[0] * invAway, y = away[1] * invAway, m = away[2] * invAway;
        dir[0] = x * cosine - y * sine, dir[1] = x * sine + y * cosine, dir[2] = m;
    }
    if (h->look[2] > 0 && sky) {
        REAL rgb[3] = {0, 0, 0};
        FN(starLayer)(dir[0], dir[1], dir[2], K(90.), 26, K(.1), K(1.6), rgb);
        FN(starLayer)(dir[0], dir[1], dir[2], K(240.), 70, K(.17), K(.22), rgb);
        const REAL skyTurn = FN(turnsOf)(dir[1], dir[0]);
        const REAL heightPos = (dir[2] * K(.5) + K(.5)) * (REAL)(ORACLE_SKY_HEIGHT - 1);
        const REAL skyFloor = FN(minX)(FLOOR(heightPos), (REAL)(ORACLE_SKY_HEIGHT - 2));
        const int32_t skyRow = FN(toInt)(skyFloor);
        const REAL s0 = FN(rowAt)(map, mapCount, ORACLE_SKY_AT, ORACLE_SKY_WIDTH, skyRow, skyTurn);
        const REAL s1 = FN(rowAt)(map, mapCount, ORACLE_SKY_AT, ORACLE_SKY_WIDTH, skyRow + 1, skyTurn);
        const REAL dust = s0 + (s1 - s0) * (heightPos - skyFloor);
        rgb[0] = rgb[0] + dust * K(.92);
        rgb[1] = rgb[1] + dust * K(.86);
        rgb[2] = rgb[2] + dust;
        REAL shown = through * h->look[2];
        if (doppler != 0) {
            const REAL g1 = (REAL)1 + doppler * (invEnergy * moved - (REAL)1);
            const REAL g2 = g1 * g1;
            shown = shown * (g2 * g2);
        }
        for (int c = 0; c < 3; ++c) sum[c] = sum[c] + rgb[c] * shown;
    }
    for (int c = 0; c < 3; ++c) out[c] = sum[c];
    if (end) {
        end->hitR = (float)hitR;
        end->hitPhi = (float)hitPhi;
        for (int c = 0; c < 3; ++c) end->dir[c] = (float)dir[c];
        end->mino = (float)mino;
        end->steps = (uint16_t)steps;
        end->crossings = (uint8_t)(crossings > 255 ? 255 : crossings);
        end->kind = (uint8_t)(kind | (lit ? ORACLE_LIT : 0));
        end->fp64Steps = 0;
        end->reserved = 0;
    }
}

#undef K
#undef FN
#undef CAT
#undef CAT_
