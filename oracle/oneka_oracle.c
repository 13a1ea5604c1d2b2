/*
 * oneka_oracle.c -- CPU FP64 restatement of OnekaPy's tracking and chronicle
 * path.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU
 * baseline leg of bench.py call it as the checker.  The product never links
 * or calls it.
 *
 * Every expression keeps the reference's left-to-right evaluation order.  The
 * file must be compiled with -ffp-contract=off so that no multiply-add is
 * fused, because Python float and NumPy scalar arithmetic never fuses.  The
 * reference's `x**2` and `x**(1/5)` go through libm pow(), so this file calls
 * pow() at the same places.  One documented exception is numpy.linalg.norm of
 * a 2-vector: NumPy's OpenBLAS ddot fuses it to sqrt(fma(y, y, x*x)).
 *
 * Functions follow (paths within the OnekaPy project):
 *   orc_potential          oneka/model.py:207-237 (+ 240-266 wells only)
 *   orc_discharge          oneka/model.py:269-315
 *   orc_head               oneka/model.py:318-350
 *   orc_velocity           oneka/model.py:353-389 (general)
 *                          oneka/model.py:392-427 (confined)
 *   orc_backtrace          oneka/capturezone.py:127-253 (Dormand-Prince 5(4))
 *   orc_insert             oneka/probabilityfield.py:264-310
 *   orc_distancesquared    oneka/probabilityfield.py:380-427
 *   orc_track              oneka/capturezone.py:51-123 + probabilityfield.py:313-372
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* One realization of the flow model: Model(base, K, n, H, wells, xo, yo, coef). */
typedef struct {
    double base, conductivity, porosity, thickness;
    double xo, yo;
    double coef[6];
    int32_t nwells;
    int32_t pad;
    const double *xw, *yw, *qw;      /* wells in list order */
} OrcModel;

enum { ORC_OK = 0, ORC_DRY = 1, ORC_STEP_LIMIT = 2 };

static double py_sq(double x) { return pow(x, 2.0); }  /* Python/NumPy x**2 */

double orc_potential_wells(const OrcModel* m, double x, double y)
{
    double potential = 0.0;
    for (int i = 0; i < m->nwells; ++i) {
        double dx = x - m->xw[i];
        double dy = y - m->yw[i];
        double r2 = dx * dx + dy * dy;
        potential += m->qw[i] * log(r2) * 0.07957747154594767;
    }
    return potential;
}

double orc_potential(const OrcModel* m, double x, double y)
{
    double dx = x - m->xo;
    double dy = y - m->yo;
    double potential = (m->coef[0] * py_sq(dx) + m->coef[1] * py_sq(dy)
                        + m->coef[2] * dx * dy
                        + m->coef[3] * dx + m->coef[4] * dy
                        + m->coef[5]);
    potential += orc_potential_wells(m, x, y);
    return potential;
}

void orc_discharge(const OrcModel* m, double x, double y, double* qx, double* qy)
{
    double dx = x - m->xo;
    double dy = y - m->yo;
    double Qx = -(2.0 * m->coef[0] * dx + m->coef[2] * dy + m->coef[3]);
    double Qy = -(2.0 * m->coef[1] * dy + m->coef[2] * dx + m->coef[4]);
    for (int i = 0; i < m->nwells; ++i) {
        dx = x - m->xw[i];
        dy = y - m->yw[i];
        double r2 = dx * dx + dy * dy;
        Qx += -m->qw[i] * dx / r2 * 0.15915494309189535;
        Qy += -m->qw[i] * dy / r2 * 0.15915494309189535;
    }
    *qx = Qx;
    *qy = Qy;
}

/* Returns ORC_DRY where the reference raises AquiferError. */
int orc_head(const OrcModel* m, double x, double y, double* head)
{
    double potential = orc_potential(m, x, y);
    if (potential <= 0) return ORC_DRY;
    if (potential < 0.5 * m->conductivity * py_sq(m->thickness))
        *head = sqrt(2.0 * potential / m->conductivity);
    else
        *head = ((potential + 0.5 * m->conductivity * py_sq(m->thickness))
                 / (m->conductivity * m->thickness));
    return ORC_OK;
}

int orc_velocity(const OrcModel* m, double x, double y, int confined, double* vx, double* vy)
{
    double Qx, Qy;
    orc_discharge(m, x, y, &Qx, &Qy);
    if (confined) {
        *vx = Qx / (m->thickness * m->porosity);
        *vy = Qy / (m->thickness * m->porosity);
        return ORC_OK;
    }
    double head;
    if (orc_head(m, x, y, &head) != ORC_OK) return ORC_DRY;
    if (head <= 0) return ORC_DRY;
    if (head > m->thickness) {
        *vx = Qx / (m->thickness * m->porosity);
        *vy = Qy / (m->thickness * m->porosity);
    } else {
        *vx = Qx / (head * m->porosity);
        *vy = Qy / (head * m->porosity);
    }
    return ORC_OK;
}

/* The backtracing feval closure, oneka/stochastic.py:253-260: returns -V. */
static int feval(const OrcModel* m, int confined, const double* xy, double* k)
{
    double vx, vy;
    int s = orc_velocity(m, xy[0], xy[1], confined, &vx, &vy);
    if (s != ORC_OK) return s;
    k[0] = -vx;
    k[1] = -vy;
    return ORC_OK;
}

/* Output sink for the vertices of one trace. */
typedef struct {
    double* xy;          /* [cap][2] or NULL */
    int64_t cap;
    int64_t n;           /* vertices produced (may exceed cap) */
    double bbox[4];      /* xmin, xmax, ymin, ymax over all vertices */
} OrcTrace;

static void trace_push(OrcTrace* tr, double x, double y)
{
    if (tr->xy && tr->n < tr->cap) {
        tr->xy[2 * tr->n] = x;
        tr->xy[2 * tr->n + 1] = y;
    }
    if (tr->n == 0) {
        tr->bbox[0] = tr->bbox[1] = x;
        tr->bbox[2] = tr->bbox[3] = y;
    } else {
        if (x < tr->bbox[0]) tr->bbox[0] = x;
        if (x > tr->bbox[1]) tr->bbox[1] = x;
        if (y < tr->bbox[2]) tr->bbox[2] = y;
        if (y > tr->bbox[3]) tr->bbox[3] = y;
    }
    tr->n++;
}

/* Python's min(a, b, c): the first argument wins unless a later one is strictly smaller. */
static double py_min3(double a, double b, double c)
{
    double m = a;
    if (b < m) m = b;
    if (c < m) m = c;
    return m;
}

/*
 * Dormand-Prince backtrace, oneka/capturezone.py:198-253.  Vertices are the
 * release point followed by every accepted point.  A dry cell ends the trace
 * with the vertices so far (the reference's bare except, :249-253).  The
 * attempt cap (max_attempts <= 0 disables it) stands in for the reference's
 * endless loop on a NaN velocity.
 */
int orc_backtrace(const OrcModel* m, int confined, double xs, double ys,
                  double duration, double tol, double maxstep, int64_t max_attempts,
                  OrcTrace* tr, int64_t* naccept, int64_t* nattempt)
{
    const double EPS = 2.220446049250313e-16;
    const double a2 = 1.0 / 5.0;
    const double a31 = 3.0 / 40.0, a32 = 9.0 / 40.0;
    const double a41 = 44.0 / 45.0, a42 = -56.0 / 15.0, a43 = 32.0 / 9.0;
    const double a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0,
                 a54 = -212.0 / 729.0;
    const double a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0,
                 a64 = 49.0 / 176.0, a65 = -5103.0 / 18656.0;
    const double a71 = 35.0 / 384.0, a73 = 500.0 / 1113.0, a74 = 125.0 / 192.0,
                 a75 = -2187.0 / 6784.0, a76 = 11.0 / 84.0;
    const double e1 = 71.0 / 57600.0, e2 = -1.0 / 40.0, e3 = -71.0 / 16695.0,
                 e4 = 71.0 / 1920.0, e5 = -17253.0 / 339200.0, e6 = 22.0 / 525.0;

    double t = 0.0;
    double sgn = (duration > 0) ? 1.0 : ((duration < 0) ? -1.0 : 0.0);
    double dt = 0.1 * sgn;
    double xy[2] = {xs, ys};
    double k1[2], k2[2], k3[2], k4[2], k5[2], k6[2], p[2], xyt[2];
    int64_t acc = 0, att = 0;
    int status = ORC_OK;

    trace_push(tr, xs, ys);
    if (feval(m, confined, xy, k1) != ORC_OK) { status = ORC_DRY; goto done; }

    while (fabs(t) < fabs(duration)) {
        if (max_attempts > 0 && att >= max_attempts) { status = ORC_STEP_LIMIT; break; }
        att++;
        if (fabs(t + dt) > fabs(duration)) dt = duration - t;

        for (int c = 0; c < 2; ++c) p[c] = xy[c] + dt * (a2 * k1[c]);
        if (feval(m, confined, p, k2) != ORC_OK) { status = ORC_DRY; break; }
        for (int c = 0; c < 2; ++c) p[c] = xy[c] + dt * (a31 * k1[c] + a32 * k2[c]);
        if (feval(m, confined, p, k3) != ORC_OK) { status = ORC_DRY; break; }
        for (int c = 0; c < 2; ++c) p[c] = xy[c] + dt * (a41 * k1[c] + a42 * k2[c] + a43 * k3[c]);
        if (feval(m, confined, p, k4) != ORC_OK) { status = ORC_DRY; break; }
        for (int c = 0; c < 2; ++c)
            p[c] = xy[c] + dt * (a51 * k1[c] + a52 * k2[c] + a53 * k3[c] + a54 * k4[c]);
        if (feval(m, confined, p, k5) != ORC_OK) { status = ORC_DRY; break; }
        for (int c = 0; c < 2; ++c)
            p[c] = xy[c] + dt * (a61 * k1[c] + a62 * k2[c] + a63 * k3[c] + a64 * k4[c] + a65 * k5[c]);
        if (feval(m, confined, p, k6) != ORC_OK) { status = ORC_DRY; break; }
        for (int c = 0; c < 2; ++c)
            xyt[c] = xy[c] + dt * (a71 * k1[c] + a73 * k3[c] + a74 * k4[c] + a75 * k5[c] + a76 * k6[c]);
        /* FSAL: the reference stores f(xyt) in k2 (:236). */
        if (feval(m, confined, xyt, k2) != ORC_OK) { status = ORC_DRY; break; }
        double err0 = dt * (e1 * k1[0] + e2 * k2[0] + e3 * k3[0] + e4 * k4[0] + e5 * k5[0] + e6 * k6[0]);
        double err1 = dt * (e1 * k1[1] + e2 * k2[1] + e3 * k3[1] + e4 * k4[1] + e5 * k5[1] + e6 * k6[1]);
        double a0 = fabs(err0), a1 = fabs(err1);
        /* numpy inf-norm: max(|.|), NaN propagating */
        double est = (isnan(a0) || isnan(a1)) ? NAN : (a1 > a0 ? a1 : a0);
        double d0 = xyt[0] - xy[0], d1 = xyt[1] - xy[1];
        double ds = sqrt(fma(d1, d1, d0 * d0));

        if ((est < tol) && (ds < maxstep)) {
            t = t + dt;
            k1[0] = k2[0];
            k1[1] = k2[1];
            xy[0] = xyt[0];
            xy[1] = xyt[1];
            trace_push(tr, xy[0], xy[1]);
            acc++;
        }
        dt = 0.9 * py_min3(pow(tol / (est + EPS), 1.0 / 5.0), maxstep / (ds + EPS), 10.0) * dt;
    }
done:
    if (naccept) *naccept = acc;
    if (nattempt) *nattempt = att;
    return status;
}

/* ProbabilityField.distancesquared, oneka/probabilityfield.py:407-427. */
double orc_distancesquared(double ax, double ay, double bx, double by, double cx, double cy)
{
    double bax = bx - ax;
    double bay = by - ay;
    double cax = cx - ax;
    double cay = cy - ay;
    double perpdot = bax * cay - bay * cax;
    double dot = bax * cax + bay * cay;
    double length2 = bax * bax + bay * bay;
    double alpha2 = perpdot * perpdot / length2;
    double beta2 = dot * dot / length2;
    double d2;
    if (dot < 0)
        d2 = alpha2 + beta2;
    else if (beta2 > length2)
        d2 = alpha2 + beta2 - 2 * dot + length2;
    else
        d2 = alpha2;
    return d2;
}

/*
 * Node grid: node (i, j) sits at (xmin + j*dx, ymin + i*dy); row-major uint8
 * marks.  The frame of a particle (xmin/ymin of the grid the reference held
 * when that trace was rasterized, and its offset inside this grid) lets the
 * caller replay the auto-expanding grid exactly; a fixed window uses
 * coff = roff = 0 and the grid's own extent.
 */
typedef struct {
    double xmin, ymin, dx, dy;
    int32_t nrows, ncols;
} OrcGrid;

typedef struct {
    double xmin, ymin;       /* grid origin at the time of rasterization */
    int32_t coff, roff;      /* column/row of that origin inside the full grid */
    int32_t ncols, nrows;    /* extent at that time */
} OrcFrame;

static double py_min2(double a, double b) { return (b < a) ? b : a; }
static double py_max2(double a, double b) { return (b > a) ? b : a; }

/* ProbabilityField.insert, oneka/probabilityfield.py:296-310. */
void orc_insert(const OrcGrid* g, const OrcFrame* f, uint8_t* rgrid,
                double ax, double ay, double bx, double by, double umbra)
{
    double umbra_squared = umbra * umbra;
    double fl = floor((py_min2(ax, bx) - umbra - f->xmin) / g->dx);
    double fr = floor((py_max2(ax, bx) + umbra - f->xmin) / g->dx) + 1;
    double fb = floor((py_min2(ay, by) - umbra - f->ymin) / g->dy);
    double ft = floor((py_max2(ay, by) + umbra - f->ymin) / g->dy) + 1;
    if (!(fl < (double)f->ncols) || !(fr > 0) || !(fb < (double)f->nrows) || !(ft > 0)) return;
    int64_t left = fl < 0 ? 0 : (int64_t)fl;
    int64_t right = fr > f->ncols ? f->ncols : (int64_t)fr;
    int64_t bottom = fb < 0 ? 0 : (int64_t)fb;
    int64_t top = ft > f->nrows ? f->nrows : (int64_t)ft;
    for (int64_t j = left; j < right; ++j) {
        for (int64_t i = bottom; i < top; ++i) {
            int64_t gi = i + f->roff, gj = j + f->coff;
            if (gi < 0 || gi >= g->nrows || gj < 0 || gj >= g->ncols) continue;
            uint8_t* cell = &rgrid[gi * (int64_t)g->ncols + gj];
            if (!*cell) {
                double cx = f->xmin + (double)j * g->dx;
                double cy = f->ymin + (double)i * g->dy;
                if (orc_distancesquared(ax, ay, bx, by, cx, cy) < umbra_squared) *cell = 1;
            }
        }
    }
}

/* ProbabilityField.rasterize without the expand (the caller fixes the frame). */
void orc_rasterize(const OrcGrid* g, const OrcFrame* f, uint8_t* rgrid,
                   const double* xy, int64_t n, double umbra)
{
    for (int64_t i = 0; i + 1 < n; ++i)
        orc_insert(g, f, rgrid, xy[2 * i], xy[2 * i + 1], xy[2 * i + 2], xy[2 * i + 3], umbra);
}

/*
 * Track options shared by every particle of the batch.
 */
typedef struct {
    double duration, tol, maxstep, umbra;
    int32_t confined;
    int32_t pad;
    int64_t max_attempts;
} OrcOpts;

/*
 * Batched restatement of compute_capturezone + register for nreal
 * realizations (oneka/capturezone.py:113-123, oneka/probabilityfield.py:342-359).
 *
 *   wells_xy   [nwells][2]           well positions (list order)
 *   coef       [nreal][6], q [nreal][nwells], aquifer [nreal][3] = (K, n, H)
 *   rskip      [nreal] or NULL       nonzero: realization not tracked/registered
 *   release    [npaths][2]
 *   frames     [nreal][npaths] or NULL (fixed window)
 *   counts     [nrows][ncols] int32, incremented once per realization per marked node
 *   per-particle outputs (each may be NULL): naccept, nattempt, status [nreal][npaths],
 *   endpoint [nreal][npaths][2], bbox [nreal][npaths][4],
 *   vertices [nreal][npaths][max_vertices][2] with nvertices [nreal][npaths].
 * Returns the number of registered realizations.
 */
int64_t orc_track(const double* wells_xy, int32_t nwells, double base, double xo, double yo,
                  const double* coef, const double* q, const double* aquifer, const int32_t* rskip,
                  int32_t nreal, const double* release, int32_t npaths, const OrcOpts* o,
                  const OrcGrid* g, const OrcFrame* frames, int32_t* counts,
                  int32_t* naccept, int32_t* nattempt, int32_t* status, double* endpoint,
                  double* bbox, double* vertices, int64_t max_vertices, int64_t* nvertices,
                  int32_t nthreads)
{
    int64_t registered = 0;
    int64_t cells = (int64_t)g->nrows * g->ncols;
    double* xw = (double*)malloc(sizeof(double) * (nwells > 0 ? nwells : 1));
    double* yw = (double*)malloc(sizeof(double) * (nwells > 0 ? nwells : 1));
    for (int i = 0; i < nwells; ++i) { xw[i] = wells_xy[2 * i]; yw[i] = wells_xy[2 * i + 1]; }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif

#pragma omp parallel reduction(+ : registered)
    {
        uint8_t* rgrid = counts ? (uint8_t*)calloc((size_t)cells, 1) : NULL;
        int64_t vcap = 4096;
        double* vbuf = (double*)malloc(sizeof(double) * 2 * vcap);
#pragma omp for schedule(dynamic, 1)
        for (int32_t r = 0; r < nreal; ++r) {
            if (rskip && rskip[r]) continue;
            OrcModel m;
            m.base = base;
            m.conductivity = aquifer[3 * r + 0];
            m.porosity = aquifer[3 * r + 1];
            m.thickness = aquifer[3 * r + 2];
            m.xo = xo;
            m.yo = yo;
            for (int c = 0; c < 6; ++c) m.coef[c] = coef[6 * (int64_t)r + c];
            m.nwells = nwells;
            m.xw = xw;
            m.yw = yw;
            m.qw = q + (int64_t)r * nwells;
            for (int32_t p = 0; p < npaths; ++p) {
                int64_t idx = (int64_t)r * npaths + p;
                OrcTrace tr;
                memset(&tr, 0, sizeof(tr));
                for (;;) {
                    tr.xy = vbuf;
                    tr.cap = vcap;
                    tr.n = 0;
                    int64_t acc, att;
                    int s = orc_backtrace(&m, o->confined, release[2 * p], release[2 * p + 1],
                                          o->duration, o->tol, o->maxstep, o->max_attempts,
                                          &tr, &acc, &att);
                    if (tr.n > vcap) {             /* grow and redo: traces are deterministic */
                        vcap = tr.n * 2;
                        vbuf = (double*)realloc(vbuf, sizeof(double) * 2 * vcap);
                        continue;
                    }
                    if (naccept) naccept[idx] = (int32_t)acc;
                    if (nattempt) nattempt[idx] = (int32_t)att;
                    if (status) status[idx] = s;
                    break;
                }
                if (endpoint) {
                    endpoint[2 * idx] = vbuf[2 * (tr.n - 1)];
                    endpoint[2 * idx + 1] = vbuf[2 * (tr.n - 1) + 1];
                }
                if (bbox) memcpy(&bbox[4 * idx], tr.bbox, sizeof(tr.bbox));
                if (nvertices) nvertices[idx] = tr.n;
                if (vertices) {
                    int64_t nv = tr.n < max_vertices ? tr.n : max_vertices;
                    memcpy(&vertices[2 * idx * max_vertices], vbuf, sizeof(double) * 2 * nv);
                }
                if (rgrid) {
                    OrcFrame fixed = {g->xmin, g->ymin, 0, 0, g->ncols, g->nrows};
                    const OrcFrame* f = frames ? &frames[idx] : &fixed;
                    orc_rasterize(g, f, rgrid, vbuf, tr.n, o->umbra);
                }
            }
            if (rgrid) {
                for (int64_t c = 0; c < cells; ++c) {
                    if (rgrid[c]) {
#pragma omp atomic
                        counts[c] += 1;
                        rgrid[c] = 0;
                    }
                }
            }
            registered += 1;
        }
        free(vbuf);
        free(rgrid);
    }
    free(xw);
    free(yw);
    return registered;
}

/* Pointwise model evaluation for the known-answer tests (oneka/model.py). */
void orc_evaluate(const double* wells_xy, const double* q, int32_t nwells, double base,
                  double K, double n, double H, double xo, double yo, const double* coef,
                  const double* pts, int64_t npts, double* potential, double* discharge,
                  double* head, double* velocity, int32_t* status, int32_t confined)
{
    double* xw = (double*)malloc(sizeof(double) * (nwells > 0 ? nwells : 1));
    double* yw = (double*)malloc(sizeof(double) * (nwells > 0 ? nwells : 1));
    for (int i = 0; i < nwells; ++i) { xw[i] = wells_xy[2 * i]; yw[i] = wells_xy[2 * i + 1]; }
    OrcModel m = {base, K, n, H, xo, yo, {0}, nwells, 0, xw, yw, q};
    for (int c = 0; c < 6; ++c) m.coef[c] = coef[c];
    for (int64_t i = 0; i < npts; ++i) {
        double x = pts[2 * i], y = pts[2 * i + 1];
        potential[i] = orc_potential(&m, x, y);
        orc_discharge(&m, x, y, &discharge[2 * i], &discharge[2 * i + 1]);
        double h = NAN;
        int s = orc_head(&m, x, y, &h);
        head[i] = h;
        double vx = NAN, vy = NAN;
        s = orc_velocity(&m, x, y, confined, &vx, &vy);
        velocity[2 * i] = vx;
        velocity[2 * i + 1] = vy;
        status[i] = s;
    }
    free(xw);
    free(yw);
}
