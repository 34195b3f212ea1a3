/*
 * FP32 C + OpenMP restatement of synkrotomo's projection + SIRT path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker for "the reference's FP32
 * behaviour" and the timed CPU stand-in for the reference (whose Futhark
 * compiler is not available to build the reference itself).  The product
 * never links or calls it.
 *
 * The code follows the reference's Futhark programs step by step, in float32,
 * with the same evaluation order of every expression (compile with
 * -ffp-contract=off so no multiply-add is fused):
 *   futhark/sirtlib.fut            preprocess / fix_projections / postprocess_fp
 *   futhark/forwardprojection.fut  fp / forwardprojection / main
 *   futhark/backprojection.fut     intersect_fact / bp / backprojection / main
 *   futhark/SIRT.fut               SIRT / main
 *   futhark/SIRT3D.fut             main (intended semantics)
 * The outer `map`s are OpenMP `parallel for` loops (the loop Futhark's
 * multicore backend parallelises); every `reduce (+)` is a sequential loop in
 * index order, as the Futhark C backends evaluate it.
 *
 * One deliberate difference: the reference reads the sinogram unchecked in
 * the backprojector (backprojection.fut:64).  Here a detector index outside
 * [0, numrhos) contributes nothing and is counted (cpuref_last_oob).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    float cost, sint, lbase;
} line_t;

static int64_t g_last_oob = 0;

/* ---------------- sirtlib.fut ---------------- */

/* sirtlib.fut:6-7 */
static int is_flat(float c, float s) { return fabsf(s) >= fabsf(c); }

/* sirtlib.fut:9-10 */
static float safe_inverse(float v) { return v == 0.0f ? 0.0f : 1.0f / v; }

/* sirtlib.fut:28-44.  Fills the steep lines and the flat lines (each in
 * original angle order, as Futhark's stable `partition`), the per-angle flat
 * flag and angle_index = steep indices ++ flat indices (line 42). */
static void preprocess(const float *angles, int a, line_t *steep, int *nsteep,
                       line_t *flat, int *nflat, int *angle_index, unsigned char *flatflag) {
    int ns = 0, nf = 0;
    for (int i = 0; i < a; i++) {
        float c = cosf(angles[i]);
        float s = sinf(angles[i]);
        float q1 = s / c, q2 = c / s;
        float lsteep = sqrtf(1.0f + q1 * q1);   /* line 33: (sin/cos)**2 */
        float lflat = sqrtf(1.0f + q2 * q2);    /* line 34 */
        int f = is_flat(c, s);
        flatflag[i] = (unsigned char)f;
        if (f) {
            flat[nf].cost = -s; flat[nf].sint = c; flat[nf].lbase = lflat;   /* line 41 */
            nf++;
        } else {
            steep[ns].cost = c; steep[ns].sint = -s; steep[ns].lbase = lsteep; /* line 41 */
            ns++;
        }
    }
    int k = 0;
    for (int i = 0; i < a; i++) if (!flatflag[i]) angle_index[k++] = i;
    for (int i = 0; i < a; i++) if (flatflag[i]) angle_index[k++] = i;
    *nsteep = ns;
    *nflat = nf;
}

/* sirtlib.fut:16-21: stable partition of the sinogram rows into (steep, flat). */
static void fix_projections(const float *proj, int a, int numrhos, const unsigned char *flatflag,
                            float *steep, float *flat) {
    int64_t ks = 0, kf = 0;
    for (int i = 0; i < a; i++) {
        const float *row = proj + (int64_t)i * numrhos;
        if (flatflag[i]) { memcpy(flat + kf, row, sizeof(float) * numrhos); kf += numrhos; }
        else { memcpy(steep + ks, row, sizeof(float) * numrhos); ks += numrhos; }
    }
}

/* image transpose (forwardprojection.fut:80-82, SIRT.fut:28-30, backprojection.fut:75-77) */
static void transpose(const float *in, float *out, int size) {
#pragma omp parallel for schedule(static)
    for (int r = 0; r < size; r++)
        for (int c = 0; c < size; c++) out[(int64_t)c * size + r] = in[(int64_t)r * size + c];
}

/* ---------------- forwardprojection.fut ---------------- */

/* forwardprojection.fut:21-59 */
static void fp(const line_t *lines, int nl, float rhozero, float deltarho, int numrhos, int halfsize,
               const float *img, float *out) {
    const int size = halfsize * 2;
    const int pixindexcorrection = halfsize * (1 + size);
#pragma omp parallel for collapse(2) schedule(static)
    for (int li = 0; li < nl; li++) {
        for (int r = 0; r < numrhos; r++) {
            const float cost = lines[li].cost, sint = lines[li].sint, lbase = lines[li].lbase;
            const float slope = -sint / cost;                   /* line 26 */
            const float rho = rhozero + (float)r * deltarho;    /* line 28 */
            const float intercept = rho / cost;                 /* line 29 */
            float acc = 0.0f;
            for (int i = -halfsize; i < halfsize; i++) {
                const float xbot = (float)i * slope + intercept;          /* 32 */
                const float xtop = xbot + slope;                          /* 33 */
                const int xpixbot = (int)floorf(xbot);                    /* 35 */
                const int xpixtop = (int)floorf(xtop);                    /* 36 */
                const float xpixmax = (float)(xpixbot > xpixtop ? xpixbot : xpixtop); /* 38 */
                const float xdiff = xtop - xbot;                          /* 40 */
                const int single = xpixbot == xpixtop;                    /* 42 */
                const int botin = xpixbot >= -halfsize && xpixbot < halfsize;              /* 43 */
                const int topin = (!single) && xpixtop >= -halfsize && xpixtop < halfsize; /* 44 */
                const float lxbotfac = (xpixmax - xbot) / xdiff;          /* 46 */
                const float lxbot = single ? lbase : lxbotfac * lbase;    /* 47 */
                const float lxtop = ((xtop - xpixmax) / xdiff) * lbase;   /* 48 */
                const int pixbot = xpixbot + i * size + pixindexcorrection; /* 50 */
                const int pixtop = xpixtop + i * size + pixindexcorrection; /* 51 */
                const float bot = botin ? lxbot * img[pixbot] : 0.0f;     /* 53 */
                const float top = topin ? lxtop * img[pixtop] : 0.0f;     /* 54 */
                acc += bot + top;                                         /* 31, 56 */
            }
            out[(int64_t)li * numrhos + r] = acc;
        }
    }
}

/* forwardprojection.fut:71-84 (with sirtlib.fut:24-25 postprocess_fp) */
int cpuref_forwardprojection(const float *angles, int a, float rhozero, float deltarho, int numrhos,
                             const float *image, int64_t n, float *out) {
    const int size = (int)sqrtf((float)n);   /* line 76 */
    const int halfsize = size / 2;           /* line 77 */
    line_t *steep = malloc(sizeof(line_t) * (a + 1)), *flat = malloc(sizeof(line_t) * (a + 1));
    int *angle_index = malloc(sizeof(int) * (a + 1));
    unsigned char *ff = malloc(a + 1);
    float *imageT = malloc(sizeof(float) * (size_t)n);
    float *vals = malloc(sizeof(float) * (size_t)a * numrhos + 4);
    if (!steep || !flat || !angle_index || !ff || !imageT || !vals) return 1;
    int ns, nf;
    preprocess(angles, a, steep, &ns, flat, &nf, angle_index, ff);
    transpose(image, imageT, size);
    fp(steep, ns, rhozero, deltarho, numrhos, halfsize, image, vals);
    fp(flat, nf, rhozero, deltarho, numrhos, halfsize, imageT, vals + (int64_t)ns * numrhos);
    /* postprocess_fp: scatter (steep ++ flat) back to angle-major order */
    for (int k = 0; k < a; k++)
        memcpy(out + (int64_t)angle_index[k] * numrhos, vals + (int64_t)k * numrhos, sizeof(float) * numrhos);
    free(steep); free(flat); free(angle_index); free(ff); free(imageT); free(vals);
    return 0;
}

/* ---------------- backprojection.fut ---------------- */

/* backprojection.fut:22-33 */
static float intersect_fact(float plus, float minus, float mini, float maxi) {
    const float lo = fmaxf(plus - mini, 0.0f);
    const float hi = fmaxf(maxi - minus, 0.0f);
    const float diff = plus - minus;
    const float inside = fminf(lo, hi);
    const float prop = inside == 0.0f ? 0.0f : inside / diff;
    return fminf(prop, 1.0f);
}

/* backprojection.fut:36-68 */
static int64_t bp(const line_t *lines, int nl, float rhozero, float deltarho, int rpp, int numrhos,
                  int halfsize, const float *proj, float *out) {
    const float fact = sqrtf(2.0f) / 2.0f;   /* line 20 */
    const int size = halfsize * 2;
    int64_t oob = 0;
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : oob)
    for (int irow = -halfsize; irow < halfsize; irow++) {
        for (int icol = -halfsize; icol < halfsize; icol++) {
            const float xmin = (float)icol, ymin = (float)irow;   /* 46-47 */
            float acc = 0.0f;
            for (int idx = 0; idx < nl; idx++) {
                const float cost = lines[idx].cost, sint = lines[idx].sint, lbase = lines[idx].lbase;
                const float slope = -sint / cost;                                /* 49 */
                const float x = xmin + 0.5f - fact * cost;                       /* 50 */
                const float y = ymin + 0.5f - fact * sint;
                const float rho = cost * x + sint * y;                           /* 51 */
                const float s = ceilf((rho - rhozero) / deltarho);               /* 53 */
                const float xbase = ymin * slope;                                /* 54 */
                float accl = 0.0f;
                for (int i = 0; i < rpp; i++) {
                    const float sprime = s + (float)i;                           /* 56 */
                    const float r = sprime * deltarho + rhozero;                 /* 57 */
                    const float xbot = xbase + (r / cost);                       /* 58 */
                    const float xtop = xbot + slope;                             /* 59 */
                    const float maxx = fmaxf(xbot, xtop), minx = fminf(xbot, xtop);
                    const float l = intersect_fact(maxx, minx, xmin, xmin + 1.0f) * lbase; /* 62 */
                    const int sp = (int)sprime;
                    float v = 0.0f;
                    if (sp >= 0 && sp < numrhos) v = proj[(int64_t)idx * numrhos + sp];  /* 63-64 */
                    else if (l != 0.0f) oob++;
                    accl += l * v;
                }
                acc += accl;
            }
            out[(int64_t)(irow + halfsize) * size + (icol + halfsize)] = acc;
        }
    }
    return oob;
}

/* backprojection.fut:70-78 */
static int64_t backprojection(const float *steep_proj, const float *flat_proj, const line_t *steep, int ns,
                              const line_t *flat, int nf, float rhozero, float deltarho, int rpp, int numrhos,
                              int halfsize, float *out, float *tmp1, float *tmp2) {
    const int size = halfsize * 2;
    int64_t oob = bp(steep, ns, rhozero, deltarho, rpp, numrhos, halfsize, steep_proj, out);
    oob += bp(flat, nf, rhozero, deltarho, rpp, numrhos, halfsize, flat_proj, tmp1);
    transpose(tmp1, tmp2, size);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)size * size; i++) out[i] = out[i] + tmp2[i];
    return oob;
}

static int rhos_per_pixel(float deltarho) { return (int)ceilf(sqrtf(2.0f) / deltarho); }  /* 87 */

/* backprojection.fut:82-93 */
int cpuref_backprojection(const float *angles, int a, float rhozero, float deltarho, int size_in,
                          const float *projections, int64_t p, float *out) {
    const int rpp = rhos_per_pixel(deltarho);
    const int halfsize = size_in / 2;
    const int size = halfsize * 2;
    const int numrhos = (int)(p / a);
    line_t *steep = malloc(sizeof(line_t) * (a + 1)), *flat = malloc(sizeof(line_t) * (a + 1));
    int *angle_index = malloc(sizeof(int) * (a + 1));
    unsigned char *ff = malloc(a + 1);
    float *sp = malloc(sizeof(float) * (size_t)p + 4), *fpj = malloc(sizeof(float) * (size_t)p + 4);
    float *t1 = malloc(sizeof(float) * (size_t)size * size + 4), *t2 = malloc(sizeof(float) * (size_t)size * size + 4);
    if (!steep || !flat || !angle_index || !ff || !sp || !fpj || !t1 || !t2) return 1;
    int ns, nf;
    preprocess(angles, a, steep, &ns, flat, &nf, angle_index, ff);
    fix_projections(projections, a, numrhos, ff, sp, fpj);
    g_last_oob = backprojection(sp, fpj, steep, ns, flat, nf, rhozero, deltarho, rpp, numrhos, halfsize, out, t1, t2);
    free(steep); free(flat); free(angle_index); free(ff); free(sp); free(fpj); free(t1); free(t2);
    return 0;
}

/* ---------------- SIRT.fut ---------------- */

/* SIRT.fut:9-41.  `image` is the start (copied), the result goes to out. */
int cpuref_sirt(const float *angles, int a, float rhozero, float deltarho, const float *image, int64_t n,
                const float *projections, int64_t p, int iterations, float *out) {
    const int rpp = rhos_per_pixel(deltarho);   /* 15 */
    const int size = (int)sqrtf((float)n);      /* 16 */
    const int halfsize = size / 2;              /* 17 */
    const int numrhos = (int)(p / a);           /* 18 */
    /* SIRT.fut:38-39 adds a (2*halfsize)^2-pixel backprojection to the n-pixel
     * image: the shapes agree only for an even square side. */
    if (size < 2 || (size & 1) || (int64_t)size * size != n) return 2;
    line_t *steep = malloc(sizeof(line_t) * (a + 1)), *flat = malloc(sizeof(line_t) * (a + 1));
    int *angle_index = malloc(sizeof(int) * (a + 1));
    unsigned char *ff = malloc(a + 1);
    if (!steep || !flat || !angle_index || !ff) return 1;
    int ns, nf;
    preprocess(angles, a, steep, &ns, flat, &nf, angle_index, ff);   /* 19 */
    const int64_t ps = (int64_t)ns * numrhos, pf = (int64_t)nf * numrhos;
    float *steep_proj = malloc(sizeof(float) * (ps + 1)), *flat_proj = malloc(sizeof(float) * (pf + 1));
    float *rs = malloc(sizeof(float) * (ps + 1)), *rf = malloc(sizeof(float) * (pf + 1));
    float *ws = malloc(sizeof(float) * (ps + 1)), *wf = malloc(sizeof(float) * (pf + 1));
    float *ones = malloc(sizeof(float) * (size_t)n), *colinv = malloc(sizeof(float) * (size_t)n);
    float *x = malloc(sizeof(float) * (size_t)n), *xT = malloc(sizeof(float) * (size_t)n);
    float *bpv = malloc(sizeof(float) * (size_t)n), *t1 = malloc(sizeof(float) * (size_t)n), *t2 = malloc(sizeof(float) * (size_t)n);
    if (!steep_proj || !flat_proj || !rs || !rf || !ws || !wf || !ones || !colinv || !x || !xT || !bpv || !t1 || !t2) return 1;
    fix_projections(projections, a, numrhos, ff, steep_proj, flat_proj);   /* 20 */
    for (int64_t i = 0; i < n; i++) ones[i] = 1.0f;
    fp(steep, ns, rhozero, deltarho, numrhos, halfsize, ones, rs);          /* 22 */
    fp(flat, nf, rhozero, deltarho, numrhos, halfsize, ones, rf);           /* 23 */
    for (int64_t i = 0; i < ps; i++) rs[i] = safe_inverse(rs[i]);
    for (int64_t i = 0; i < pf; i++) rf[i] = safe_inverse(rf[i]);
    for (int64_t i = 0; i < ps; i++) ws[i] = 1.0f;
    for (int64_t i = 0; i < pf; i++) wf[i] = 1.0f;
    g_last_oob = backprojection(ws, wf, steep, ns, flat, nf, rhozero, deltarho, rpp, numrhos, halfsize, colinv, t1, t2); /* 25 */
    for (int64_t i = 0; i < n; i++) colinv[i] = safe_inverse(colinv[i]);
    memcpy(x, image, sizeof(float) * (size_t)n);
    for (int it = 0; it < iterations; it++) {                                /* 27 */
        transpose(x, xT, size);                                              /* 28-30 */
        fp(steep, ns, rhozero, deltarho, numrhos, halfsize, x, ws);          /* 31 */
        fp(flat, nf, rhozero, deltarho, numrhos, halfsize, xT, wf);          /* 32 */
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < ps; i++) ws[i] = rs[i] * (steep_proj[i] - ws[i]);   /* 33, 35 */
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < pf; i++) wf[i] = rf[i] * (flat_proj[i] - wf[i]);    /* 34, 36 */
        g_last_oob += backprojection(ws, wf, steep, ns, flat, nf, rhozero, deltarho, rpp, numrhos, halfsize, bpv, t1, t2); /* 37 */
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) x[i] = x[i] + colinv[i] * bpv[i];          /* 38-39 */
    }
    memcpy(out, x, sizeof(float) * (size_t)n);
    free(steep); free(flat); free(angle_index); free(ff); free(steep_proj); free(flat_proj);
    free(rs); free(rf); free(ws); free(wf); free(ones); free(colinv); free(x); free(xT); free(bpv); free(t1); free(t2);
    return 0;
}

/* SIRT3D.fut:18-29, intended semantics: `size` slices from a zero start; the
 * reference's `rhos` array becomes rhozero = rhos[0],
 * deltarho = rhos[1] - rhos[0] (archive/projection_lib.fut:114-115).
 * `nslices` slices are reconstructed (the reference uses size). */
int cpuref_sirt3d(const float *angles, int a, const float *rhos, int r, const float *projections,
                  int iterations, int size, int nslices, float *out) {
    const float rhozero = rhos[0];
    const float deltarho = r > 1 ? rhos[1] - rhozero : 1.0f;
    const int64_t n = (int64_t)size * size;
    if (size < 2 || (size & 1)) return 2;
    float *zero = calloc((size_t)n, sizeof(float));
    if (!zero) return 1;
    for (int i = 0; i < nslices; i++) {
        int rc = cpuref_sirt(angles, a, rhozero, deltarho, zero, n, projections + (int64_t)i * r * a,
                             (int64_t)r * a, iterations, out + (int64_t)i * n);
        if (rc) { free(zero); return rc; }
    }
    free(zero);
    return 0;
}

int64_t cpuref_last_oob(void) { return g_last_oob; }

int cpuref_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}
