/*
 * rl_oracle.c -- CPU FP64 restatement of RADLite's line-raytrace path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the parity checker for the GPU path: it is
 * imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and
 * nothing in the product (radlite_gb300/, include/) links or calls it.
 *
 * Parity pinning: the reference ships no tests, golden outputs or known-answer vectors
 * for this path, and its Fortran cannot be compiled in this container (no Fortran
 * compiler), so this restatement is "parity unpinned" by the reference itself. It is
 * pinned instead by analytic known-answer cases (tests/test_oracle_kat.py) and by the
 * committed fixtures under tests/golden/ that record its own outputs.
 *
 * It follows, function by function (file:line in RADLITE/ of pontoppi/radlite):
 *   setup_rays_circular        telescope.F:715-1191   (imethod=1, nrref=10: main.F:37-38)
 *   make_image_circular        telescope.F:339-631    (NONREDUNDANT, configure.h:53)
 *   calc_freq_flux_observer    telescope.F:1320-1437
 *   make_trajectory_c          telescope.F:2787-3720  (LONGCHAR_EXTRA_POINTS, main.h:338)
 *   charintline                telescope.F:3889-4312
 *   get_line_dust_values       line.F:3965-4217       omega_dot_v  line.F:2650-2662
 *   clever_integrate_element_linedust line.F:4636-4848 (SUBGRID, configure.h:7)
 *   integrate_element_linedust line.F:4515-4624       voigt_profile line.F:2280-2314
 *   qdr_src_2                  transfer.F:1498-1571
 *   line_setup_passband        line.F:427-545         prepare_lines line.F:1708-1823
 *   line_dust_compute_src_alp  line.F:3502-3677       bplanck setup.F:937-952
 *   line_init_passband_starbc  line.F:3797-3845       aksmax line.F:2968-3218
 *   header/write_line_spectrum telescope.F:1662-1804
 *   readers: grid.F:711-819,1098-1210; setup.F:159-235,295-670,754-919,1453-1690;
 *            dust.F:92-447; star.F:449-569; source.F:494-543; line.F:142-367,811-950,
 *            1826-1985,3918-3935; telescope.F:86-257; main.F:488-686; tools.F:6-20
 *   bracketing search: own bisection with the guess-then-bisect semantics of hunt
 *   (nrecip.F:157-197); extra-point ordering: own stable insertion sort.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <ctype.h>
#include "rl_oracle.h"

#define PI_ 3.1415926535897932385
#define TEL_EPS 1.0e-10
#define LEVTHRES 1.0e-3
#define RAYADPT 4
#define RAYRNPT 4
#define RAYEXPT 100

/* ----------------------------------------------------------------------------------- */
/* error handling                                                                        */
/* ----------------------------------------------------------------------------------- */
static char g_err[512];
static int fail(const char* fmt, ...) {
    va_list ap; va_start(ap, fmt); vsnprintf(g_err, sizeof g_err, fmt, ap); va_end(ap);
    return -1;
}
const char* rlo_last_error(void) { return g_err; }

/* ----------------------------------------------------------------------------------- */
/* Fortran-style record input: list-directed reads consume whole records               */
/* ----------------------------------------------------------------------------------- */
typedef struct { char* buf; size_t n, pos; } frec;

static int fr_open(frec* f, const char* dir, const char* name) {
    char path[1024]; snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE* fp = fopen(path, "rb");
    if (!fp) return fail("cannot open %s", path);
    fseek(fp, 0, SEEK_END); long n = ftell(fp); fseek(fp, 0, SEEK_SET);
    f->buf = (char*)malloc((size_t)n + 2); f->n = (size_t)n; f->pos = 0;
    if (fread(f->buf, 1, (size_t)n, fp) != (size_t)n) { fclose(fp); return fail("read error %s", path); }
    f->buf[n] = '\n'; f->buf[n + 1] = 0; fclose(fp);
    return 0;
}
static int fr_exists(const char* dir, const char* name) {
    char path[1024]; snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE* fp = fopen(path, "rb"); if (fp) { fclose(fp); return 1; } return 0;
}
static void fr_close(frec* f) { free(f->buf); f->buf = NULL; }

/* Read the next record (line) into out; returns 0 at EOF. */
static int fr_line(frec* f, char* out, size_t cap) {
    if (f->pos >= f->n) return 0;
    size_t i = 0;
    while (f->pos < f->n && f->buf[f->pos] != '\n') {
        char c = f->buf[f->pos++];
        if (c != '\r' && i + 1 < cap) out[i++] = c;
    }
    if (f->pos < f->n) f->pos++;
    out[i] = 0; return 1;
}

/* List-directed read of ntok items, spanning records; rest of the last record dropped. */
static int fr_list(frec* f, int ntok, char toks[][96]) {
    int got = 0; char line[4096];
    while (got < ntok) {
        if (!fr_line(f, line, sizeof line)) return fail("unexpected end of file");
        char* p = line;
        while (*p && got < ntok) {
            while (*p == ' ' || *p == '\t' || *p == ',') p++;
            if (!*p) break;
            int k = 0;
            while (*p && *p != ' ' && *p != '\t' && *p != ',') { if (k < 95) toks[got][k++] = *p; p++; }
            toks[got][k] = 0; got++;
        }
    }
    return 0;
}
static int tok_d(const char* t, double* v) {
    char b[96]; strncpy(b, t, 95); b[95] = 0;
    for (char* q = b; *q; q++) if (*q == 'd' || *q == 'D') *q = 'e';
    char* e; *v = strtod(b, &e);
    if (e == b) return fail("not a number: '%s'", t);
    if (*e == '+' || *e == '-') {   /* Fortran exponent without a letter */
        char* e2; long ex = strtol(e, &e2, 10);
        if (e2 != e + 1 && *e2 == 0) { *v *= pow(10.0, (double)ex); return 0; }
    }
    if (*e != 0) return fail("not a number: '%s'", t);
    return 0;
}
static int rd_d(frec* f, double* v) { char t[1][96]; if (fr_list(f, 1, t)) return -1; return tok_d(t[0], v); }
static int rd_i(frec* f, int* v) { double d; if (rd_d(f, &d)) return -1; *v = (int)d; return 0; }
static int rd_s(frec* f, char* s, size_t cap) {
    char t[1][96]; if (fr_list(f, 1, t)) return -1; strncpy(s, t[0], cap - 1); s[cap - 1] = 0; return 0;
}
static int rd_dn(frec* f, int n, double* v) {  /* n values, list-directed across records */
    char line[1 << 16]; int got = 0;
    while (got < n) {
        if (!fr_line(f, line, sizeof line)) return fail("unexpected end of file");
        char* p = line;
        while (*p && got < n) {
            while (*p == ' ' || *p == '\t' || *p == ',') p++;
            if (!*p) break;
            char* q = p; while (*q && *q != ' ' && *q != '\t' && *q != ',') q++;
            char save = *q; *q = 0;
            if (tok_d(p, &v[got])) return -1;
            got++; *q = save; p = q;
        }
    }
    return 0;
}
/* Fixed-column numeric field (Fortran Fw.d / Ew.d / Iw input, blanks ignored). */
static double col_num(const char* line, int start, int width, int d) {
    char b[64]; int k = 0; int len = (int)strlen(line);
    int has_dot = 0;
    for (int i = start; i < start + width && i < len; i++) {
        char c = line[i];
        if (c == ' ' || c == '\t') continue;
        if (c == 'd' || c == 'D') c = 'e';
        if (c == '.') has_dot = 1;
        if (k < 63) b[k++] = c;
    }
    b[k] = 0;
    if (k == 0) return 0.0;
    double v = strtod(b, NULL);
    if (!has_dot && d > 0) {   /* implied decimal point applies to the mantissa */
        char* e = strpbrk(b, "eE+-");
        if (e == b && (b[0] == '+' || b[0] == '-')) e = strpbrk(b + 1, "eE+-");
        if (e) { double ex = strtod(e + (e[0] == 'e' || e[0] == 'E'), NULL); *e = 0; v = strtod(b, NULL) * pow(10.0, -d) * pow(10.0, ex); }
        else v = v * pow(10.0, -d);
    }
    return v;
}

/* ----------------------------------------------------------------------------------- */
/* bracketing search with the index rules of hunt (nrecip.F:157-197), xx 1-based xx[1..n]: */
/* with "past j" = x >= xx[j] (x < xx[j] for a descending table), bracket [lo, hi] from the */
/* guess by probes at distances 2^i - 1 (upwards while past, downwards while not past),    */
/* then lo + the count of nodes strictly inside the bracket with x > xx[j] (x <= xx[j]    */
/* descending). An exact hit on a node the bracket stopped on returns that node, one      */
/* strictly inside returns the node below it.                                            */
/* ----------------------------------------------------------------------------------- */
static int node_past(const double* xx, int asc, double x, int j) { return asc ? x >= xx[j] : x < xx[j]; }
static int node_before(const double* xx, int asc, double x, int j) { return asc ? x < xx[j] : x >= xx[j]; }
static int node_beyond(const double* xx, int asc, double x, int j) { return asc ? x > xx[j] : x <= xx[j]; }

static int hunt1(const double* xx, int n, double x, int guess) {
    int asc = xx[n] > xx[1];
    int lo = 0, hi = n + 1;
    if (guess >= 1 && guess <= n) {
        int step;
        if (node_past(xx, asc, x, guess)) {
            lo = guess;
            for (step = 1; guess + step <= n; step = 2 * step + 1) {
                if (!node_past(xx, asc, x, guess + step)) { hi = guess + step; break; }
                lo = guess + step;
            }
        } else {
            hi = guess;
            for (step = 1; guess - step >= 1; step = 2 * step + 1) {
                if (!node_before(xx, asc, x, guess - step)) { lo = guess - step; break; }
                hi = guess - step;
            }
        }
    }
    /* nodes lo+1 .. hi-1 that x lies beyond precede the others: bisect for their count */
    int a = lo, b = hi;   /* beyond(a) or a == lo; not beyond(b) or b == hi */
    while (b - a > 1) {
        int m = a + (b - a) / 2;
        if (node_beyond(xx, asc, x, m)) a = m; else b = m;
    }
    return a;
}

/* hunt1 for tests: the table xx0[0..n-1] as xx[1..n] */
int rlo_hunt(const double* xx0, int n, double x, int guess) { return hunt1(xx0 - 1, n, x, guess); }

/* ----------------------------------------------------------------------------------- */
/* model                                                                                 */
/* ----------------------------------------------------------------------------------- */
struct rlo_model {
    int nr, nth, ny;
    double* Rg;     /* R(ix), ix=-1..nr+2 -> Rg[ix+1] */
    double* Tg;     /* TH(iy), iy=-1..ny+2 -> Tg[iy+1] */
    int* ridx;      /* ridx_it(it), it=-4..ny+4 -> ridx[it+4] */
    double *rho, *vel, *lw, *abun;  /* cell = (ir-1)*nth + (it-1); vel[3*cell+c] */
    int nspec, nsize[4];
    double* drho;   /* [ispec][cell] */
    double* dtemp;  /* [ispec][isize][cell] */
    int ncont; double* cnu; double* kabs; double* ksca;  /* kabs[(ispec*4+isize)*ncont+i] */
    double* scat;   /* [ifreq][cell] or NULL */
    int nlev; double* pop;  /* [cell][lev] */
    double *Ecm, *g, *Eerg;
    int nlin; int *lup, *ldn; double *Aud, *lfreq;
    double umass;
    double rstar; double* starcont; int starpump;
    double* isrf;   /* [1..ncont] interstellfield.inp (outer boundary 3), else NULL */
    int maser;      /* masing found by the last line image or position-velocity cube */
    long long overshoot;   /* quadrature overshoots of the last line image or cube */
    int outer_bc, inner_bc, line_dust;
    /* camera & passband */
    double incl_rad; int nphi, dbdr, nrext;
    double vmax, dv, radvelo; int nlspec, ilstart, style, nfr;
    int command;                                   /* 0 spectrum, 2 position-velocity cube */
    int pv_nx, pv_ny, pv_addstar; double pv_szx, pv_szy, pv_phioff, pv_xoff, pv_yoff;
    char molname[96], molfile[200];
    double aksmax;
    /* rays */
    int nrays, nrr; double *x0, *z0, *rays_r, *ri; double theta0;
    /* per-line dust tables */
    double *ldsrc, *ldalp;  /* [line][cell] */
};

#define RG(m, ix) ((m)->Rg[(ix) + 1])
#define TG(m, iy) ((m)->Tg[(iy) + 1])
#define RIDX(m, it) ((m)->ridx[(it) + 4])
#define CELL(m, ir, it) (((ir) - 1) * (m)->nth + ((it) - 1))

void rlo_free(rlo_model* m) {
    if (!m) return;
    void* ptrs[] = {m->Rg, m->Tg, m->ridx, m->rho, m->vel, m->lw, m->abun, m->drho, m->dtemp, m->cnu,
                    m->kabs, m->ksca, m->scat, m->pop, m->Ecm, m->g, m->Eerg, m->lup, m->ldn, m->Aud,
                    m->lfreq, m->starcont, m->isrf, m->x0, m->z0, m->rays_r, m->ri, m->ldsrc, m->ldalp};
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) free(ptrs[i]);
    free(m);
}

static double bplanck(double temp, double nu) {
    if (temp == 0.0) return 0.0;
    return 1.47455e-47 * nu * nu * nu / (exp(4.7989e-11 * nu / temp) - 1.0) + 1.0e-290;
}

/* scalar field "nr nt imirt" then ir-outer, it-inner values (setup.F:1584-1690) */
static int read_scalar(const char* dir, const char* name, rlo_model* m, double* out) {
    frec f; if (fr_open(&f, dir, name)) return -1;
    char t[3][96]; int rc = fr_list(&f, 3, t);
    if (!rc) {
        double a, b, c; tok_d(t[0], &a); tok_d(t[1], &b); tok_d(t[2], &c);
        if ((int)c == 0) rc = fail("%s: theta mirroring flag must be 1", name);
        else if ((int)a != m->nr || 2 * (int)b != m->ny) rc = fail("%s: inconsistent dimensions", name);
    }
    for (int i = 0; !rc && i < m->nr * m->nth; i++) rc = rd_d(&f, &out[i]);
    fr_close(&f); return rc;
}

static int read_model(const char* dir, rlo_model* m) {
    frec f; char s[200];
    /* radlite.inp (main.F:488-686, setup.F:1117-1137), comment lines dropped and records
       cut to 16 characters as strip_comments does (tools.F:6-20) */
    {
        frec raw; if (fr_open(&raw, dir, "radlite.inp")) return -1;
        size_t cap = raw.n + 64; char* nb = (char*)malloc(cap); size_t k = 0; char line[4096];
        while (fr_line(&raw, line, sizeof line)) {
            if (line[0] == '#' || line[0] == ';' || line[0] == '%' || line[0] == '=') continue;
            line[16] = 0; size_t L = strlen(line);
            memcpy(nb + k, line, L); k += L; nb[k++] = '\n';
        }
        fr_close(&raw); f.buf = nb; f.n = k; f.pos = 0; nb[k] = 0;
        int fmt, idum; double ddum, incl;
        int rc = rd_i(&f, &fmt);
        if (!rc && fmt < 100) rc = fail("radlite.inp format %d not supported", fmt);
        if (!rc) rc = rd_i(&f, &idum) || rd_i(&f, &idum);
        if (!rc && fmt >= 103) rc = rd_i(&f, &idum);
        if (!rc) rc = rd_d(&f, &ddum) || rd_i(&f, &idum) || rd_i(&f, &idum);
        for (int i = 0; !rc && i < 6; i++) rc = rd_d(&f, &ddum);   /* angular grid setup */
        if (!rc) rc = rd_i(&f, &m->outer_bc) || rd_i(&f, &m->inner_bc) || rd_i(&f, &idum);
        if (!rc) rc = rd_d(&f, &incl) || rd_i(&f, &m->nphi) || rd_i(&f, &m->dbdr) || rd_i(&f, &m->nrext);
        for (int i = 0; !rc && i < 4; i++) rc = rd_i(&f, &idum);
        if (!rc && fmt >= 101) rc = rd_i(&f, &idum);
        if (!rc && fmt >= 102) rc = rd_i(&f, &idum);
        if (!rc) rc = rd_i(&f, &idum);
        if (!rc && fmt >= 104) rc = rd_i(&f, &idum);
        int wp = 0, dodust = 0, doline = 0;
        if (!rc) rc = rd_i(&f, &wp);
        if (!rc && wp != -551) rc = fail("radlite.inp: setup type %d not supported", wp);
        if (!rc) rc = rd_i(&f, &dodust) || rd_i(&f, &doline) || rd_i(&f, &m->line_dust) || rd_i(&f, &m->starpump);
        fr_close(&f);
        if (rc) return -1;
        if (m->nrext == 0) return fail("radlite.inp: nrrayextra must be non-zero");
        if (dodust != 0 || doline == 0) return fail("radlite.inp: only line transfer is supported");
        m->inner_bc = 2;   /* forced by setup -551 (setup.F:1135) */
        if (m->outer_bc != 0 && m->outer_bc != 2 && m->outer_bc != 3)
            return fail("outer boundary type %d not supported", m->outer_bc);
    }
    /* radius.inp / theta.inp (grid.F:711-819, 1098-1210) */
    if (fr_open(&f, dir, "radius.inp")) return -1;
    if (rd_i(&f, &m->nr)) return -1;
    if (m->nr < 3) return fail("radius.inp: need at least 3 points");
    m->Rg = (double*)calloc((size_t)m->nr + 4, sizeof(double));
    for (int ix = 1; ix <= m->nr; ix++) if (rd_d(&f, &m->Rg[ix + 1])) return -1;
    fr_close(&f);
    int nr = m->nr;
    RG(m, 0) = RG(m, 1) * RG(m, 1) / RG(m, 2);
    RG(m, -1) = RG(m, 0) * RG(m, 0) / RG(m, 1);
    RG(m, nr + 1) = RG(m, nr) * RG(m, nr) / RG(m, nr - 1);
    RG(m, nr + 2) = RG(m, nr + 1) * RG(m, nr + 1) / RG(m, nr);
    for (int ix = 1; ix < nr; ix++)
        if (RG(m, ix + 1) / RG(m, ix) - 1.0 < 1.0e4 * TEL_EPS) return fail("radial grid too fine for the safety number");
    if (fr_open(&f, dir, "theta.inp")) return -1;
    { char t[2][96]; if (fr_list(&f, 2, t)) return -1; double a, b; tok_d(t[0], &a); tok_d(t[1], &b);
      m->nth = (int)a; if ((int)b == 0) return fail("theta.inp: mirroring flag must be 1"); }
    m->ny = 2 * m->nth;
    int ny = m->ny;
    m->Tg = (double*)calloc((size_t)ny + 4, sizeof(double));
    for (int iy = 1; iy <= m->nth; iy++) {
        if (rd_d(&f, &m->Tg[iy + 1])) return -1;
        if (TG(m, iy) > 1.5707963268 || TG(m, iy) < 0) return fail("theta.inp: theta out of range");
    }
    fr_close(&f);
    for (int iy = 1; iy <= m->nth; iy++) TG(m, 2 * m->nth + 1 - iy) = 3.14159265359 - TG(m, iy);
    TG(m, 0) = -TG(m, 1); TG(m, -1) = -TG(m, 2);
    TG(m, ny + 1) = (double)(2.0f * 3.1415926f) - TG(m, ny);
    TG(m, ny + 2) = (double)(2.0f * 3.1415926f) - TG(m, ny - 1);
    m->ridx = (int*)calloc((size_t)ny + 9, sizeof(int));
    for (int it = -4; it <= ny + 4; it++) {   /* interpol.F:87-100 */
        int v = it;
        if (v < 1) v = 1 - v;
        if (v > ny) v = 2 * ny + 1 - v;
        if (v > ny / 2) v = ny + 1 - v;
        RIDX(m, it) = v;
    }
    int ncell = m->nr * m->nth;
    /* frequency.inp (grid.F:1427-1482) */
    if (fr_open(&f, dir, "frequency.inp")) return -1;
    if (rd_i(&f, &m->ncont)) return -1;
    if (m->ncont < 2) return fail("frequency.inp: need at least 2 frequencies");
    m->cnu = (double*)calloc((size_t)m->ncont + 2, sizeof(double));   /* 1-based */
    for (int i = 1; i <= m->ncont; i++) if (rd_d(&f, &m->cnu[i])) return -1;
    fr_close(&f);
    /* interstellfield.inp for outer boundary 3 (read_interstellfield, star.F:690-727): the
       frequency count, then one intensity per frequency */
    if (m->outer_bc == 3) {
        if (!fr_exists(dir, "interstellfield.inp")) return fail("outer boundary type 3 needs interstellfield.inp");
        if (fr_open(&f, dir, "interstellfield.inp")) return -1;
        int nf = 0;
        if (rd_i(&f, &nf)) return -1;
        if (nf != m->ncont) return fail("interstellfield.inp: frequency count differs from frequency.inp");
        m->isrf = (double*)calloc((size_t)m->ncont + 2, sizeof(double));
        for (int i = 1; i <= m->ncont; i++) if (rd_d(&f, &m->isrf[i])) return -1;
        fr_close(&f);
    }
    /* line.inp header (line.F:142-200) */
    if (fr_open(&f, dir, "line.inp")) return -1;
    { int fmtl, nsp; if (rd_i(&f, &fmtl)) return -1; if (fmtl == 2 && rd_i(&f, &nsp)) return -1;
      if (fmtl != 1 && fmtl != 2) return fail("line.inp: format %d", fmtl);
      if (rd_d(&f, &m->umass)) return -1; }
    fr_close(&f);
    /* dust density (setup.F:681-746 via read_vector_field isep=1); dust is read only
       when it is included in the lines (setup.F:1144-1147, main.F:150-151) */
    if (m->line_dust) {
        const char* dn = fr_exists(dir, "dustdensity.inp") ? "dustdensity.inp" : "dustdens.inp";
        if (fr_open(&f, dir, dn)) return -1;
        char t[4][96]; if (fr_list(&f, 4, t)) return -1;
        double a[4]; for (int i = 0; i < 4; i++) tok_d(t[i], &a[i]);
        m->nspec = (int)a[0];
        if (m->nspec < 1 || m->nspec > 4) return fail("dust density: species count %d", m->nspec);
        if ((int)a[1] != nr || 2 * (int)a[2] != ny || (int)a[3] == 0) return fail("dust density: inconsistent dimensions");
        m->drho = (double*)calloc((size_t)m->nspec * ncell, sizeof(double));
        for (int i = 0; i < m->nspec * ncell; i++) if (rd_d(&f, &m->drho[i])) return -1;
        fr_close(&f);
    }
    /* dust temperature (setup.F:159-235 via read_vecvector_field) */
    if (m->line_dust) {
        int flnr = 0; char fn[64];
        if (fr_open(&f, dir, "dusttemp.info")) return -1;
        if (rd_i(&f, &flnr)) return -1;
        fr_close(&f);
        if (flnr == -2) strcpy(fn, "dusttemp_final.dat"); else snprintf(fn, sizeof fn, "dusttemp_%d.dat", flnr);
        if (fr_open(&f, dir, fn)) return -1;
        char t[4][96]; if (fr_list(&f, 4, t)) return -1;
        double a[4]; for (int i = 0; i < 4; i++) tok_d(t[i], &a[i]);
        if ((int)a[0] != m->nspec || (int)a[1] != nr || 2 * (int)a[2] != ny) return fail("%s: inconsistent dimensions", fn);
        m->dtemp = (double*)calloc((size_t)m->nspec * 4 * ncell, sizeof(double));
        for (int is = 0; is < m->nspec; is++) {
            int nsz; if (rd_i(&f, &nsz)) return -1;
            if (nsz < 1 || nsz > 4) return fail("%s: size count", fn);
            m->nsize[is] = nsz;
            for (int iz = 0; iz < nsz; iz++)
                for (int i = 0; i < ncell; i++) if (rd_d(&f, &m->dtemp[((size_t)is * 4 + iz) * ncell + i])) return -1;
        }
        fr_close(&f);
    }
    /* dust opacities (dust.F:92-447) */
    if (m->line_dust) {
        if (fr_open(&f, dir, "dustopac.inp")) return -1;
        int fmt, nsp; if (rd_i(&f, &fmt) || rd_i(&f, &nsp) || rd_s(&f, s, sizeof s)) return -1;
        if (nsp != m->nspec) return fail("dustopac.inp: %d species, density has %d", nsp, m->nspec);
        m->kabs = (double*)calloc((size_t)16 * (m->ncont + 2), sizeof(double));
        m->ksca = (double*)calloc((size_t)16 * (m->ncont + 2), sizeof(double));
        for (int is = 0; is < nsp; is++) {
            int mode, quantum, ifile; double dd;
            if (rd_i(&f, &mode)) return -1;
            if (fmt >= 2) { if (rd_i(&f, &quantum)) return -1;
                if (quantum == 2) { if (rd_d(&f, &dd)) return -1; }
                else if (quantum == 3) { if (rd_d(&f, &dd) || rd_d(&f, &dd)) return -1; } }
            if (rd_i(&f, &ifile)) return -1;
            if (mode == -2) { if (rd_d(&f, &dd) || rd_d(&f, &dd)) return -1; }
            else if (mode == -3) { for (int q = 0; q < 4; q++) if (rd_d(&f, &dd)) return -1; }
            else if (mode != -1) return fail("dustopac.inp: read mode %d not supported", mode);
            char fn[64]; snprintf(fn, sizeof fn, "dustopac_%d.inp", ifile);
            frec g2; if (fr_open(&g2, dir, fn)) return -1;
            char t[2][96]; if (fr_list(&g2, 2, t)) return -1;
            double a0, a1; tok_d(t[0], &a0); tok_d(t[1], &a1);
            /* "-1 nfreq", then "nsize idum ntemp" and ntemp tables each after its temperature
               range (read_dustopac_file, dust.F:320-480, built with DUST_OPAC_TEMPDEP); the
               line dust uses the first table only (dust_kappawgt_abs(.,1,.,.), line.F:3582) */
            int nfq = (int)a0, nsz = (int)a1, ntemp = 1, trange = (int)a0 == -1;
            if (trange) {
                char t3[3][96]; if (fr_list(&g2, 3, t3)) return -1;
                double b0, b1, b2; tok_d(t3[0], &b0); tok_d(t3[1], &b1); tok_d(t3[2], &b2);
                nfq = nsz; nsz = (int)b0; ntemp = (int)b2;
                if (ntemp < 1) return fail("%s: temperature range count must be positive", fn);
            }
            if (nfq != m->ncont) return fail("%s: frequency count mismatch", fn);
            if (nsz != m->nsize[is]) return fail("%s: size count mismatch", fn);
            double bold = 0.0, dv;
            for (int itp = 0; itp < ntemp; itp++) {
                if (trange) {
                    char t2[2][96]; double ta, tb;
                    if (fr_list(&g2, 2, t2)) return -1;
                    tok_d(t2[0], &ta); tok_d(t2[1], &tb);
                    if (ta < bold) return fail("%s: temperature ranges overlap", fn);
                    if (fabs((ta - bold) / (ta + bold)) > 1.0e-3) return fail("%s: gap between temperature ranges", fn);
                    if (ta < 0.0 || tb < 0.0 || tb < ta) return fail("%s: invalid temperature range", fn);
                    bold = tb;
                }
                for (int i = 1; i <= m->ncont; i++) for (int iz = 0; iz < nsz; iz++) {
                    if (rd_d(&g2, &dv)) return -1;
                    if (itp == 0) m->kabs[((size_t)is * 4 + iz) * (m->ncont + 2) + i] = dv;
                }
                for (int i = 1; i <= m->ncont; i++) for (int iz = 0; iz < nsz; iz++) {
                    if (rd_d(&g2, &dv)) return -1;
                    if (itp == 0) m->ksca[((size_t)is * 4 + iz) * (m->ncont + 2) + i] = dv;
                }
            }
            fr_close(&g2);
            if (rd_s(&f, s, sizeof s)) return -1;
        }
        fr_close(&f);
    }
    /* optional scattering source (source.F:494-543): ifreq, it, ir(inner) */
    if (m->line_dust && fr_exists(dir, "scatsource.dat")) {
        if (fr_open(&f, dir, "scatsource.dat")) return -1;
        char t[4][96]; if (fr_list(&f, 4, t)) return -1;
        m->scat = (double*)calloc((size_t)(m->ncont + 2) * ncell, sizeof(double));
        for (int i = 1; i <= m->ncont; i++) for (int it = 1; it <= m->nth; it++) for (int ir = 1; ir <= nr; ir++) {
            double v; if (rd_d(&f, &v)) return -1; m->scat[(size_t)i * ncell + CELL(m, ir, it)] += v; }
        fr_close(&f);
    }
    /* gas fields */
    m->rho = (double*)calloc(ncell, sizeof(double));
    m->abun = (double*)calloc(ncell, sizeof(double));
    m->vel = (double*)calloc((size_t)3 * ncell, sizeof(double));
    m->lw = (double*)calloc(ncell, sizeof(double));
    if (read_scalar(dir, "density.inp", m, m->rho)) return -1;
    if (fr_exists(dir, "abundance.inp")) {   /* setup.F:864-919 */
        if (fr_open(&f, dir, "abundance.inp")) return -1;
        char t[2][96]; if (fr_list(&f, 2, t)) return -1;
        double a, b; tok_d(t[0], &a); tok_d(t[1], &b);
        if ((int)a != nr || (int)b != m->nth) return fail("abundance.inp: inconsistent dimensions");
        for (int i = 0; i < ncell; i++) { char u[2][96]; if (fr_list(&f, 2, u) || tok_d(u[0], &m->abun[i])) return -1; }
        fr_close(&f);
    } else return fail("abundance.inp is required");
    if (fr_exists(dir, "velocity.inp")) {    /* setup.F:754-789 */
        if (fr_open(&f, dir, "velocity.inp")) return -1;
        char t[2][96]; if (fr_list(&f, 2, t)) return -1;
        double a, b; tok_d(t[0], &a); tok_d(t[1], &b);
        if ((int)a != nr || (int)b != m->nth) return fail("velocity.inp: inconsistent dimensions");
        for (int i = 0; i < ncell; i++) if (rd_dn(&f, 3, &m->vel[3 * i])) return -1;
        fr_close(&f);
    }
    if (fr_exists(dir, "turbulence.inp")) {  /* setup.F:803-850 */
        if (fr_open(&f, dir, "turbulence.inp")) return -1;
        int ifm; if (rd_i(&f, &ifm)) return -1;
        char t[2][96]; if (fr_list(&f, 2, t)) return -1;
        double a, b; tok_d(t[0], &a); tok_d(t[1], &b);
        if ((int)a != nr || (int)b != m->nth) return fail("turbulence.inp: inconsistent dimensions");
        for (int i = 0; i < ncell; i++) if (rd_d(&f, &m->lw[i])) return -1;
        fr_close(&f);
    } else return fail("turbulence.inp is required (the line width)");
    /* linespectrum.inp (telescope.F:86-257) */
    {
        if (fr_open(&f, dir, "linespectrum.inp")) return -1;
        int fmt, ftel, fobj, cmd; double dist, inc;
        if (rd_i(&f, &fmt)) return -1;
        m->style = 0;
        if (fmt == 1 && rd_i(&f, &m->style)) return -1;
        if (fmt < 0 || fmt > 1) return fail("linespectrum.inp: format %d", fmt);
        if (rd_s(&f, s, sizeof s) || rd_i(&f, &ftel)) return -1;
        if (ftel != 2) return fail("linespectrum.inp: telescope format %d", ftel);
        if (rd_s(&f, s, sizeof s) || rd_d(&f, &m->vmax) || rd_d(&f, &m->dv) || rd_s(&f, s, sizeof s)) return -1;
        if (rd_i(&f, &fobj)) return -1;
        if (fobj != 2) return fail("linespectrum.inp: object format %d not supported", fobj);
        if (rd_s(&f, s, sizeof s)) return -1;
        char* d = strstr(s, ".dat");
        if (!d) return fail("linespectrum.inp: molecule file name must end with .dat");
        d[4] = 0; snprintf(m->molfile, sizeof m->molfile, "%s", s);
        size_t nlen = (size_t)(d - s); memcpy(m->molname, s, nlen); m->molname[nlen] = 0;
        if (rd_i(&f, &cmd) || rd_d(&f, &dist) || rd_d(&f, &inc) || rd_d(&f, &m->radvelo) ||
            rd_i(&f, &m->nlspec) || rd_i(&f, &m->ilstart)) return -1;
        if (cmd != 0 && cmd != 2) return fail("linespectrum.inp: command %d not supported", cmd);
        m->command = cmd;
        if (cmd == 2) {   /* telescope.F:190-218 */
            int sizespec;
            if (rd_i(&f, &m->pv_nx) || rd_i(&f, &m->pv_ny) || rd_i(&f, &sizespec) || rd_d(&f, &m->pv_szx) ||
                rd_d(&f, &m->pv_szy) || rd_d(&f, &m->pv_phioff) || rd_d(&f, &m->pv_xoff) || rd_d(&f, &m->pv_yoff) ||
                rd_i(&f, &m->pv_addstar)) return -1;
            /* 0 (arcsec): the reference warns and reads the sizes as for 1 (telescope.F:207-216) */
            if (sizespec != 0 && sizespec != 1) return fail("linespectrum.inp: size specifier %d unknown", sizespec);
        }
        m->incl_rad = inc * 0.0174532925199;
        fr_close(&f);
    }
    /* moldata.dat (line.F:1826-1985): fixed columns */
    {
        if (fr_open(&f, dir, m->molfile)) return -1;
        char line[512];
        if (rd_s(&f, s, sizeof s) || rd_s(&f, s, sizeof s) || rd_s(&f, s, sizeof s)) return -1;
        if (!fr_line(&f, line, sizeof line)) return fail("moldata: eof"); /* (F4.1) weight */
        if (rd_s(&f, s, sizeof s)) return -1;
        if (!fr_line(&f, line, sizeof line)) return fail("moldata: eof");
        m->nlev = (int)col_num(line, 0, 6, 0);
        if (m->nlev < 2) return fail("moldata: need at least 2 levels");
        if (rd_s(&f, s, sizeof s)) return -1;
        m->Ecm = (double*)calloc((size_t)m->nlev + 1, sizeof(double));
        m->g = (double*)calloc((size_t)m->nlev + 1, sizeof(double));
        m->Eerg = (double*)calloc((size_t)m->nlev + 1, sizeof(double));
        for (int i = 1; i <= m->nlev; i++) {
            if (!fr_line(&f, line, sizeof line)) return fail("moldata: eof in levels");
            m->Ecm[i] = col_num(line, 5, 12, 4); m->g[i] = col_num(line, 17, 7, 1);
            m->Eerg[i] = 1.986468498e-16 * m->Ecm[i];
        }
        if (rd_s(&f, s, sizeof s)) return -1;
        if (!fr_line(&f, line, sizeof line)) return fail("moldata: eof");
        m->nlin = (int)col_num(line, 0, 6, 0);
        if (m->nlin < 1) return fail("moldata: need at least 1 line");
        if (rd_s(&f, s, sizeof s)) return -1;
        m->lup = (int*)calloc((size_t)m->nlin + 1, sizeof(int)); m->ldn = (int*)calloc((size_t)m->nlin + 1, sizeof(int));
        m->Aud = (double*)calloc((size_t)m->nlin + 1, sizeof(double)); m->lfreq = (double*)calloc((size_t)m->nlin + 1, sizeof(double));
        for (int i = 1; i <= m->nlin; i++) {
            if (!fr_line(&f, line, sizeof line)) return fail("moldata: eof in lines");
            m->lup[i] = (int)col_num(line, 5, 5, 0); m->ldn[i] = (int)col_num(line, 10, 5, 0);
            m->Aud[i] = col_num(line, 15, 12, 3);
        }
        fr_close(&f);
        for (int i = 1; i <= m->nlin; i++) {
            if (m->lup[i] < 1 || m->ldn[i] < 1 || m->lup[i] > m->nlev || m->ldn[i] > m->nlev || m->lup[i] <= m->ldn[i])
                return fail("moldata: line %d has invalid levels", i);
            m->lfreq[i] = 1.509160e26 * (m->Eerg[m->lup[i]] - m->Eerg[m->ldn[i]]);
            if (m->lfreq[i] == 0.0) return fail("moldata: zero line frequency");
        }
        if (m->ilstart < 1 || m->ilstart + m->nlspec - 1 > m->nlin) return fail("linespectrum.inp: non-existing line requested");
        m->ilstart = 1;   /* main.F:204: the run starts at line 1 whatever the file asked */
    }
    /* line.inp per-line blocks are consumed by the reference but only feed unused options */
    /* level populations (line.F:811-950) */
    {
        int fnr; char fn[200];
        if (fr_open(&f, dir, "levelpop.info")) return -1;
        if (rd_i(&f, &fnr)) return -1;
        if (fnr == -3) {   /* line.F:847-870 */
            if (rd_s(&f, s, sizeof s)) return -1;
            if (strncmp(s, "levelpop_", 9) != 0 || !strstr(s + 9, ".dat")) return fail("levelpop.info: bad file name '%s'", s);
        }
        fr_close(&f);
        if (fnr == -1) strcpy(fn, "levelpop.dat");
        else if (fnr == -2) strcpy(fn, "levelpop_final.dat");
        else if (fnr == -3) snprintf(fn, sizeof fn, "levelpop_%s.dat", m->molname);
        else snprintf(fn, sizeof fn, "levelpop_%d.dat", fnr);
        if (fr_open(&f, dir, fn)) return -1;
        char t[4][96]; if (fr_list(&f, 4, t)) return -1;
        double a[4]; for (int i = 0; i < 4; i++) tok_d(t[i], &a[i]);
        if ((int)a[0] != nr || (int)a[1] != m->nth || (int)a[3] != 1) return fail("%s: inconsistent dimensions", fn);
        int nl = (int)a[2];
        if (nl < 2) return fail("%s: level count", fn);
        m->nlev = nl;   /* the level-population file sets nlevels (line.F:912) */
        double* tmp = (double*)malloc(sizeof(double) * (size_t)nl);
        if (rd_dn(&f, nl, tmp) || rd_dn(&f, nl, tmp)) return -1;
        free(tmp);
        m->pop = (double*)calloc((size_t)ncell * nl, sizeof(double));
        for (int c = 0; c < ncell; c++) if (rd_dn(&f, nl, &m->pop[(size_t)c * nl])) return -1;
        fr_close(&f);
        for (int i = 1; i <= m->nlin; i++)   /* prepare_lines checks every line (line.F:1734-1745) */
            if (m->lup[i] > m->nlev || m->ldn[i] > m->nlev) return fail("line %d outside the level populations", i);
    }
    /* star (star.F:449-569, line.F:3797-3845); the spectrum is read only with star pumping */
    if (fr_exists(dir, "starinfo.inp")) {
        if (fr_open(&f, dir, "starinfo.inp")) return -1;
        int ifm; if (rd_i(&f, &ifm) || rd_d(&f, &m->rstar)) return -1; fr_close(&f);
    } else m->rstar = RG(m, 1) * 1.0e-3;
    m->starcont = (double*)calloc((size_t)m->ncont + 2, sizeof(double));
    if (m->starpump != 0) {
        if (fr_exists(dir, "starspec.inp")) {
            if (fr_open(&f, dir, "starspec.inp")) return -1;
            int n; if (rd_i(&f, &n)) return -1;
            if (n != m->ncont) return fail("starspec.inp: frequency count mismatch");
            for (int i = 1; i <= n; i++) if (rd_d(&f, &m->starcont[i])) return -1;
            fr_close(&f);
        } else {
            if (fr_open(&f, dir, "starspectrum.inp")) return -1;
            int n; if (rd_i(&f, &n)) return -1;
            if (n != m->ncont) return fail("starspectrum.inp: frequency count mismatch");
            for (int i = 1; i <= n; i++) {
                char t[2][96]; double fq, fl;
                if (fr_list(&f, 2, t) || tok_d(t[0], &fq) || tok_d(t[1], &fl)) return -1;
                if (fabs(fq - m->cnu[i]) / (fq + m->cnu[i]) > 1e-3) return fail("starspectrum.inp: frequencies differ from frequency.inp");
                m->starcont[i] = 3.0308410e36 * fl / (m->rstar * m->rstar);
            }
            fr_close(&f);
        }
    }
    /* aksmax over cells (line.F:2968-3218); all lines share the width */
    m->aksmax = 0.0;
    for (int i = 0; i < ncell; i++) if (m->lw[i] > m->aksmax) m->aksmax = m->lw[i];
    /* passband (main.F:205-213) */
    m->nfr = (int)(2.0 * m->vmax / m->dv + 1);
    m->vmax = 0.5 * (m->nfr - 1) * m->dv;
    if (m->nfr < 2) return fail("passband needs at least 2 channels");
    return 0;
}

/* per-(line, cell) grey dust at the line centre (line.F:3502-3677) */
static void prepare_line_dust(rlo_model* m) {
    int ncell = m->nr * m->nth;
    m->ldsrc = (double*)calloc((size_t)(m->nlin + 1) * ncell, sizeof(double));
    m->ldalp = (double*)calloc((size_t)(m->nlin + 1) * ncell, sizeof(double));
    if (!m->line_dust) return;
    for (int il = 1; il <= m->nlin; il++) {
        double freq = m->lfreq[il];
        int i = hunt1(m->cnu, m->ncont, freq, 0);
        if (i == 0 || i == m->ncont) continue;
        double wgt = (freq - m->cnu[i]) / (m->cnu[i + 1] - m->cnu[i]);
        for (int ir = 1; ir <= m->nr; ir++) for (int it = 1; it <= m->nth; it++) {
            int c = CELL(m, ir, it); double src = 0.0, alp = 0.0;
            for (int is = 0; is < m->nspec; is++) for (int iz = 0; iz < m->nsize[is]; iz++) {
                const double* ka = &m->kabs[((size_t)is * 4 + iz) * (m->ncont + 2)];
                double kw = wgt * ka[i + 1] + (1.0 - wgt) * ka[i];
                double dr = m->drho[(size_t)is * ncell + c];
                src = src + dr * kw * bplanck(m->dtemp[((size_t)is * 4 + iz) * ncell + c], freq);
                alp = alp + dr * kw;
            }
            if (m->scat) src = src + wgt * m->scat[(size_t)(i + 1) * ncell + c] + (1.0 - wgt) * m->scat[(size_t)i * ncell + c];
            for (int is = 0; is < m->nspec; is++) for (int iz = 0; iz < m->nsize[is]; iz++) {
                const double* ks = &m->ksca[((size_t)is * 4 + iz) * (m->ncont + 2)];
                double kw = wgt * ks[i + 1] + (1.0 - wgt) * ks[i];
                alp = alp + m->drho[(size_t)is * ncell + c] * kw;
            }
            m->ldsrc[(size_t)il * ncell + c] = src; m->ldalp[(size_t)il * ncell + c] = alp;
        }
    }
}

/* ray family (telescope.F:715-1191) and ring edges (telescope.F:424-488) */
static int setup_rays(rlo_model* m) {
    int nrrextra = abs(m->nrext), nrref = 10, nphi = m->nphi;
    double anginf = m->incl_rad, rstar = m->rstar;
    if (nphi < 1) return fail("nphi must be positive");
    if (m->dbdr < 1) return fail("dbdr must be positive");
    if (anginf == 0.0) return fail("inclination 0 is not representable (the reference divides by it)");
    if (fabs(anginf) < 1.0e-1) anginf = (double)0.1f * fabs(anginf) / anginf;
    m->incl_rad = anginf;
    if (rstar > RG(m, 1)) return fail("star larger than the inner grid radius");
    double theta0 = anginf + 1.0e-4, sinth0 = sin(theta0);
    m->theta0 = theta0;
    double dphi = 6.28318530718 / (1.0 * nphi), phi = 0.5 * dphi;
    double* zh = (double*)malloc(sizeof(double) * nphi); double* xh = (double*)malloc(sizeof(double) * nphi);
    for (int k = 0; k < nphi; k++) {
        zh[k] = -sin(phi) / sinth0;
        double zh02 = zh[k] * zh[k];
        double dum = 1.0 - zh02 * sinth0 * sinth0;
        dum = dum + 1.0e2 * TEL_EPS;
        if (dum < 0) { free(zh); free(xh); return fail("ray setup: negative discriminant"); }
        xh[k] = cos(phi) > 0.0 ? sqrt(dum) : -sqrt(dum);
        phi = phi + dphi;
    }
    int nrr = nrrextra + nrref + m->dbdr * (m->nr - 1);
    m->nrr = nrr; m->nrays = 1 + nrr * nphi;
    m->x0 = (double*)calloc((size_t)m->nrays + 1, sizeof(double));
    m->z0 = (double*)calloc((size_t)m->nrays + 1, sizeof(double));
    m->rays_r = (double*)calloc((size_t)nrr + 2, sizeof(double));
    m->ri = (double*)calloc((size_t)nrr + 3, sizeof(double));
    int iray = 1, irad = 1;  /* ray 1 = central: x0=z0=0 */
    double R1 = RG(m, 1), ref1 = 0.5, ref2 = 0.0;
#define PUSH_RING(rc) do { m->rays_r[irad] = (rc); for (int k = 0; k < nphi; k++) { iray++; \
        m->x0[iray] = (rc) * xh[k]; m->z0[iray] = (rc) * zh[k]; } irad++; } while (0)
    for (int ix = 1; ix <= nrrextra + nrref; ix++) {
        double rc;
        if (ix <= nrrextra) rc = ((ix - 1) * (R1 - rstar) / nrrextra) + rstar;
        else { ref2 = ref2 + ref1; ref1 = ref1 / 2; rc = ((nrrextra + ref2) * (R1 - rstar) / (nrrextra + 1.0)) + rstar; }
        PUSH_RING(rc);
    }
    for (int ix = 1; ix <= m->nr - 1; ix++) {
        double rc = RG(m, ix) * (1.0 + 1.0e3 * TEL_EPS);
        PUSH_RING(rc);
        if (m->dbdr > 1) {
            double dr = (RG(m, ix + 1) - RG(m, ix)) / (1.0 * m->dbdr);
            for (int ii = 1; ii <= m->dbdr - 1; ii++) { double rc2 = RG(m, ix) + ii * dr; PUSH_RING(rc2); }
        }
    }
#undef PUSH_RING
    free(zh); free(xh);
    double* r = m->rays_r; double* ri = m->ri;
    r[0] = 0.0; ri[0] = 0.0;
    for (int ir = 1; ir <= nrr; ir++) ri[ir] = 0.5 * (r[ir] + r[ir - 1]);
    ri[nrr + 1] = RG(m, m->nr);
    for (int ir = 1; ir <= nrr - 1; ir++)
        if (r[ir] - ri[ir] > 2 * (ri[ir + 1] - r[ir])) ri[ir] = r[ir] - 2 * (ri[ir + 1] - r[ir]);
    if (ri[1] < rstar) { if (r[1] < rstar) return fail("ray setup: internal error"); ri[1] = rstar; }
    return 0;
}

/* ----------------------------------------------------------------------------------- */
/* trajectory (telescope.F:2787-3720)                                                    */
/* ----------------------------------------------------------------------------------- */
typedef struct { int n; double *s, *r, *th, *mu, *phi, b; int *icr, *ir, *it; } traj_t;

static void sort_extra(int n, double* s, double* r, double* th, int* ir, int* it) {
    for (int i = 2; i <= n; i++) {   /* stable insertion sort on s (1-based) */
        double ks = s[i], kr = r[i], kt = th[i]; int ki = ir[i], kj = it[i]; int j = i - 1;
        while (j >= 1 && s[j] > ks) { s[j + 1] = s[j]; r[j + 1] = r[j]; th[j + 1] = th[j]; ir[j + 1] = ir[j]; it[j + 1] = it[j]; j--; }
        s[j + 1] = ks; r[j + 1] = kr; th[j + 1] = kt; ir[j + 1] = ki; it[j + 1] = kj;
    }
}

static int trajectory(const rlo_model* m, double x0, double z0, double theta0, traj_t* T) {
    const double pi = PI_, eps = TEL_EPS, epsplus = 1.0e1 * TEL_EPS;
    int nr = m->nr, ny = m->ny;
    double rrgrid[4096], ttgrid[4096];
    if (nr + 2 > 4096 || ny + 2 > 4096) return fail("grid too large for the oracle");
    for (int ix = 1; ix <= nr; ix++) rrgrid[ix] = RG(m, ix);
    for (int iy = 1; iy <= ny; iy++) ttgrid[iy] = TG(m, iy);
    double pitheta0 = 0.5 * pi - theta0;
    double costh0 = cos(theta0), sinth0 = sin(theta0);
    double costh02 = costh0 * costh0, sinth02 = sinth0 * sinth0;
    int iyeq = ny / 2, iyend = ny;
    int K = 2 * (2 * nr + ny + RAYEXPT) + 8;
    double* sar1 = (double*)malloc(sizeof(double) * K); double* sar2 = (double*)malloc(sizeof(double) * K);
    int* iyar = (int*)malloc(sizeof(int) * K);
    double* th_r = (double*)malloc(sizeof(double) * K); double* th_t = (double*)malloc(sizeof(double) * K);
    double* th_s = (double*)malloc(sizeof(double) * K); int* th_ir = (int*)malloc(sizeof(int) * K);
    int* th_it = (int*)malloc(sizeof(int) * K);
    double* r_r = (double*)malloc(sizeof(double) * K); double* r_t = (double*)malloc(sizeof(double) * K);
    double* r_s = (double*)malloc(sizeof(double) * K); int* r_ir = (int*)malloc(sizeof(int) * K);
    int* r_it = (int*)malloc(sizeof(int) * K);
    int rc = 0;
    /* theta=const crossings */
    int is = 1;
    for (int iy = 1; iy <= iyeq; iy++) {
        double theta = TG(m, iy);
        double tt = tan(theta); double tanth2 = tt * tt;
        double a = tanth2 * costh02 - sinth02;
        double b = 2.0 * tanth2 * costh0 * z0;
        double c = tanth2 * z0 * z0 - x0 * x0;
        double sd = b * b - 4.0 * a * c;
        if (sd > 0.0) {
            sd = sqrt(sd);
            iyar[is] = iy;
            sar1[is] = (-b - sd) / (2.0 * a);
            sar2[is] = (-b + sd) / (2.0 * a);
            if (sar1[is] > sar2[is]) { double d = sar1[is]; sar1[is] = sar2[is]; sar2[is] = d; }
            is++;
        }
    }
    int isnr = is - 1, isdblnr = 0;
    for (is = 1; is <= isnr; is++) if (fabs(0.5 * pi - TG(m, iyar[is])) > fabs(pitheta0)) isdblnr++;
    int iup = pitheta0 > 0.0 ? 1 : 0;
#define THR(s) sqrt(x0 * x0 + z0 * z0 + (s) * (s) + 2.0 * z0 * costh0 * (s))
#define SETTH(iss, sv, itv) do { th_r[iss] = THR(sv); th_s[iss] = (sv); th_it[iss] = (itv); th_t[iss] = TG(m, th_it[iss]); } while (0)
    if (z0 * pitheta0 > 0.0) {
        is = 1 + isdblnr;
        for (int iss = 1; iss <= isnr - isdblnr; iss++) { SETTH(iss, sar1[is], iup ? iyend + 1 - iyar[is] : iyar[is]); is++; }
        is = isnr;
        for (int iss = isnr - isdblnr + 1; iss <= 2 * isnr - 2 * isdblnr; iss++) { SETTH(iss, sar2[is], iup ? iyar[is] : iyend + 1 - iyar[is]); is--; }
        if (isdblnr > 0) {
            for (int iss = 2 * isnr + 1 - 2 * isdblnr; iss <= 2 * isnr - isdblnr; iss++) { SETTH(iss, sar1[is], iup ? iyar[is] : iyend + 1 - iyar[is]); is--; }
            is++;
            for (int iss = 2 * isnr + 1 - isdblnr; iss <= 2 * isnr; iss++) { SETTH(iss, sar2[is], iup ? iyar[is] : iyend + 1 - iyar[is]); is++; }
        }
    } else {
        is = isdblnr;
        if (isdblnr > 0) {
            for (int iss = 1; iss <= isdblnr; iss++) { SETTH(iss, sar1[is], iup ? iyend + 1 - iyar[is] : iyar[is]); is--; }
            is++;
            for (int iss = isdblnr + 1; iss <= 2 * isdblnr; iss++) { SETTH(iss, sar2[is], iup ? iyend + 1 - iyar[is] : iyar[is]); is++; }
        }
        is = isdblnr + 1;
        for (int iss = 2 * isdblnr + 1; iss <= isnr + isdblnr; iss++) { SETTH(iss, sar1[is], iup ? iyend + 1 - iyar[is] : iyar[is]); is++; }
        is = isnr;
        for (int iss = isnr + isdblnr + 1; iss <= 2 * isnr; iss++) { SETTH(iss, sar2[is], iup ? iyar[is] : iyend + 1 - iyar[is]); is--; }
    }
#undef SETTH
    int ith_amount = 2 * isnr;
    int ix = nr + 1;   /* hunt guess carried like the reference's loop variable */
    for (is = 1; is <= ith_amount; is++) {
        double r = th_r[is];
        if (r < RG(m, 1)) th_ir[is] = 0;
        else if (r > RG(m, nr)) th_ir[is] = nr;
        else { ix = hunt1(rrgrid, nr, r, ix); th_ir[is] = ix; }
    }
    /* R=const crossings */
    double bimpact = sqrt(x0 * x0 + z0 * z0 * (1.0 - costh02));
    for (ix = 1; ix <= nr; ix++) if (RG(m, ix) > bimpact) break;
    if (ix > nr) { rc = fail("trajectory outside the domain"); goto done; }
    int ir_min = ix;
    if (bimpact <= m->rstar) ir_min = 0;
    T->b = bimpact;
    int ir_amount = 2 * (nr + 1 - ir_min);
    is = 1;
    for (ix = nr; ix >= ir_min; ix--) {
        double r = (ix == 0) ? m->rstar : RG(m, ix);
        double a = 1.0, b = 2.0 * costh0 * z0, c = x0 * x0 + z0 * z0 - r * r;
        double sd = b * b - 4.0 * a * c + eps * b * b;
        if (sd < 0.0) { rc = fail("trajectory: negative discriminant"); goto done; }
        sd = sqrt(sd);
        double s1 = (-b - sd) / (2.0 * a), s2 = (-b + sd) / (2.0 * a);
        double t1 = atan(sqrt(x0 * x0 + sinth02 * s1 * s1) / (z0 + costh0 * s1)); if (t1 < 0.0) t1 += pi;
        double t2 = atan(sqrt(x0 * x0 + sinth02 * s2 * s2) / (z0 + costh0 * s2)); if (t2 < 0.0) t2 += pi;
        r_t[is] = t1; r_s[is] = s1; r_ir[is] = ix; r_r[is] = r;
        r_t[ir_amount + 1 - is] = t2; r_s[ir_amount + 1 - is] = s2; r_ir[ir_amount + 1 - is] = ix; r_r[ir_amount + 1 - is] = r;
        is++;
    }
    int iy = iyeq + 1;
    for (is = 1; is <= ir_amount; is++) { iy = hunt1(ttgrid, ny, r_t[is], iy); r_it[is] = iy; }
    int tr_amount = ir_amount + ith_amount;
    th_s[ith_amount + 1] = 1.0e30; r_s[ir_amount + 1] = 1.0e30;
    r_s[0] = -1.0e30;   /* the reference leaves r_s(0) unset; see DESIGN notes */
    double rmaxt = RG(m, nr) * (1.0 - epsplus), rmaxr = RG(m, nr) * (1.0 + epsplus);
    double rmint = RG(m, 1) * (1.0 + epsplus), rminr = RG(m, 1) * (1.0 - epsplus);
    double sbeg = -1.0e30, sprev = -1.0e30, send = 1.0e30;
    /* extra points around the r- and theta-extrema */
    double ex_s[RAYEXPT + 2], ex_r[RAYEXPT + 2], ex_t[RAYEXPT + 2]; int ex_ir[RAYEXPT + 2], ex_it[RAYEXPT + 2];
    for (int k = 0; k < RAYEXPT + 2; k++) ex_s[k] = 1.0e30;
    int isex = 1;
#define EXTH(sv) ({ double _t = atan(sqrt(x0 * x0 + sinth02 * (sv) * (sv)) / (z0 + costh0 * (sv))); if (_t < 0.0) _t += pi; _t; })
    if (bimpact > RG(m, 1)) {
        double s2 = 0.0 - z0 * costh0;
        ex_s[isex] = s2; ex_r[isex] = bimpact; ex_t[isex] = EXTH(s2);
        ex_ir[isex] = ir_min - 1;
        iy = hunt1(ttgrid, ny, ex_t[isex], iy); ex_it[isex] = iy;
        isex++;
        double s3 = s2;
        int isrt = hunt1(r_s, ir_amount, s2, 0);
        for (int irng = 1; irng <= 4; irng++) {
            double s1, sx;
            if (irng == 1) { s1 = s3; sx = r_s[isrt + 1]; }
            else if (irng == 2) { s1 = r_s[isrt]; sx = s3; }
            else if (irng == 3) { s1 = r_s[isrt + 1]; sx = (isrt + 2 <= ir_amount + 1) ? r_s[isrt + 2] : 1.0e30; }
            else { s1 = r_s[isrt - 1]; sx = r_s[isrt]; }
            double ds = (sx - s1) / (1.0 + 1.0 * RAYADPT);
            for (int iad = 1; iad <= RAYADPT; iad++) {
                double s0 = iad * ds + s1;
                ex_s[isex] = s0;
                double rr2 = sqrt(x0 * x0 + z0 * z0 + s0 * s0 + 2.0 * z0 * costh0 * s0);
                ex_r[isex] = rr2; ex_t[isex] = EXTH(s0);
                ix = hunt1(rrgrid, nr, rr2, ix); ex_ir[isex] = ix;
                iy = hunt1(ttgrid, ny, ex_t[isex], iy); ex_it[isex] = iy;
                isex++;
            }
        }
    }
    {
        double s2 = x0 * x0 * costh0 / (z0 * sinth02);
        double rr2 = sqrt(x0 * x0 + z0 * z0 + s2 * s2 + 2.0 * z0 * costh0 * s2);
        if (rr2 > RG(m, 1) && rr2 < RG(m, nr)) {
            ex_s[isex] = s2; ex_r[isex] = rr2; ex_t[isex] = EXTH(s2);
            ix = hunt1(rrgrid, nr, rr2, ix);
            if (ix == 0 || ix == nr) { rc = fail("trajectory: hunt failed at theta extremum"); goto done; }
            ex_ir[isex] = ix;
            iy = hunt1(ttgrid, ny, ex_t[isex], iy); ex_it[isex] = iy;
            isex++;
            double s3 = s2;
            int isrt = hunt1(th_s, ith_amount, s3, 0);
            if (!(isrt - RAYRNPT + 1 < 1 || isrt + RAYRNPT > ith_amount)) {
                for (int irng = 1; irng <= 4; irng++) {
                    double s1, sx;
                    if (irng == 1) { s1 = s3; sx = th_s[isrt + 1]; }
                    else if (irng == 2) { s1 = th_s[isrt]; sx = s3; }
                    else if (irng == 3) { s1 = th_s[isrt + 1]; sx = th_s[isrt + 2]; }
                    else { s1 = th_s[isrt - 1]; sx = th_s[isrt]; }
                    if (sx <= s1) { rc = fail("trajectory: theta extremum points out of order"); goto done; }
                    double ds = (sx - s1) / (1.0 + 1.0 * RAYADPT);
                    for (int iad = 1; iad <= RAYADPT; iad++) {
                        double s0 = iad * ds + s1;
                        ex_s[isex] = s0;
                        double r3 = sqrt(x0 * x0 + z0 * z0 + s0 * s0 + 2.0 * z0 * costh0 * s0);
                        ex_r[isex] = r3; ex_t[isex] = EXTH(s0);
                        ix = hunt1(rrgrid, nr, r3, ix);
                        if (ix == 0 || ix == nr) { ex_s[isex] = 1.0e30; continue; }
                        ex_ir[isex] = ix;
                        iy = hunt1(ttgrid, ny, ex_t[isex], iy); ex_it[isex] = iy;
                        isex++;
                    }
                }
            }
        }
    }
#undef EXTH
    int nrex = isex - 1;
    sort_extra(nrex, ex_s, ex_r, ex_t, ex_ir, ex_it);
    isex = 1;
    int ist = 1, isr = 1; is = 1;
    int cap = tr_amount + nrex + 2;
    T->s = (double*)malloc(sizeof(double) * cap); T->r = (double*)malloc(sizeof(double) * cap);
    T->th = (double*)malloc(sizeof(double) * cap); T->mu = (double*)malloc(sizeof(double) * cap);
    T->phi = (double*)malloc(sizeof(double) * cap);
    T->icr = (int*)malloc(sizeof(int) * cap); T->ir = (int*)malloc(sizeof(int) * cap); T->it = (int*)malloc(sizeof(int) * cap);
    for (int iss = 1; iss <= tr_amount; iss++) {
        for (;;) {
            double lim = th_s[ist] < r_s[isr] ? th_s[ist] : r_s[isr];
            if (!(ex_s[isex] < lim)) break;
            if (ex_r[isex] <= rmaxt && ex_r[isex] >= rmint && (ex_s[isex] - sprev) > eps * ex_r[isex] &&
                ex_s[isex] >= sbeg && ex_s[isex] <= send) {
                T->icr[is] = 3; T->r[is] = ex_r[isex]; T->th[is] = ex_t[isex]; T->ir[is] = ex_ir[isex];
                T->it[is] = ex_it[isex]; T->s[is] = ex_s[isex]; sprev = T->s[is]; is++;
            }
            isex++;
        }
        if (isex > RAYEXPT) { rc = fail("trajectory: too many extra points"); goto done; }
        if (th_s[ist] < r_s[isr]) {
            if (th_r[ist] <= rmaxt && th_r[ist] >= rmint && (th_s[ist] - sprev) > eps * th_r[ist] &&
                th_s[ist] >= sbeg && th_s[ist] <= send) {
                T->icr[is] = 2; T->r[is] = th_r[ist]; T->th[is] = th_t[ist]; T->ir[is] = th_ir[ist];
                T->it[is] = th_it[ist]; T->s[is] = th_s[ist]; sprev = T->s[is]; is++;
            }
            ist++;
        } else {
            if (r_r[isr] <= rmaxr && r_r[isr] >= rminr && (r_s[isr] - sprev) > eps * r_r[isr] &&
                r_s[isr] >= sbeg && r_s[isr] <= send) {
                T->icr[is] = 1; T->r[is] = r_r[isr]; T->th[is] = r_t[isr]; T->ir[is] = r_ir[isr];
                T->it[is] = r_it[isr]; T->s[is] = r_s[isr]; sprev = T->s[is]; is++;
            }
            isr++;
        }
    }
    T->n = is - 1;
    {
        double znew = z0 * sinth02, bnew = sqrt(x0 * x0 + z0 * z0 * sinth02);
        for (int k = 1; k <= T->n; k++) {
            double snew = T->s[k] + z0 * costh0;
            T->mu[k] = snew / sqrt(bnew * bnew + snew * snew);
            double q = znew + snew * costh0;
            double dummy = bnew * sqrt(bnew * bnew + snew * snew - q * q);
            double sp = dummy > 0.0 ? (bnew * bnew * costh0 - znew * snew) / dummy : epsplus;
            sp = (x0 < 0.0) ? asin(sp) : pi - asin(sp);
            while (sp < 0.0) sp += 2.0 * pi;
            while (sp >= 2.0 * pi) sp -= 2.0 * pi;
            T->phi[k] = sp;
        }
    }
done:
    free(sar1); free(sar2); free(iyar); free(th_r); free(th_t); free(th_s); free(th_ir); free(th_it);
    free(r_r); free(r_t); free(r_s); free(r_ir); free(r_it);
    return rc;
}
#undef THR

static void traj_free(traj_t* T) { free(T->s); free(T->r); free(T->th); free(T->mu); free(T->phi); free(T->icr); free(T->ir); free(T->it); }

/* ----------------------------------------------------------------------------------- */
/* the walk                                                                              */
/* ----------------------------------------------------------------------------------- */
typedef struct {
    const rlo_model* m; int il;
    double nu0abs, lfreq, Aud, Bud, Bdu, molpg;
    const double *dsrc, *dalp;
    double* dnu;   /* [1..nfr] */
    double* star;  /* [1..nfr] */
    double* isrf;  /* [1..nfr] outer-boundary start intensity (type 3), or NULL: 0 */
    long long steps;
    double tau;        /* char_tau: running optical depth of the current (ray, channel), line.F:4598 */
    int maser;         /* maserflag: some segment had line opacity x length below -0.01 */
    long long overshoot;   /* transerr_overshoot: steps whose quadrature exceeded twice theomax */
} linectx;

static int node_values(const linectx* L, int icr, int ir, int it, double dr, double dt, double mu, double phi,
                       double* srcd, double* alpd, double* dvmu, double* lw, double* nup, double* ndn) {
    const rlo_model* m = L->m;
    if (dr < 0.0 || dr > 1.0) return fail("node: dr out of range (%g)", dr);
    if (dt < 0.0 || dt > 1.0) return fail("node: dt out of range (%g)", dt);
    int r0 = ir, r1, t0, t1;
    if (dr > 0.0) { r1 = ir + 1; if (r1 > m->nr) r1 = m->nr; }
    else { r1 = ir - 1; if (r1 < 1) r1 = 1; }
    if (dt > 0.0) { t0 = it; t1 = it + 1; } else { t0 = it; t1 = it - 1; }
    t0 = RIDX(m, t0); t1 = RIDX(m, t1);
    int lu = m->lup[L->il], ld = m->ldn[L->il], nl = m->nlev;
    int c00 = CELL(m, r0, t0), c01 = CELL(m, r0, t1), c10 = CELL(m, r1, t0), c11 = CELL(m, r1, t1);
#define NU(c) (m->pop[(size_t)(c) * nl + lu - 1] * m->abun[c] * m->rho[c] * L->molpg)
#define ND(c) (m->pop[(size_t)(c) * nl + ld - 1] * m->abun[c] * m->rho[c] * L->molpg)
    double v[3];
    if (icr == 1) {
        *srcd = (1.0 - dt) * L->dsrc[c00] + dt * L->dsrc[c01];
        *alpd = (1.0 - dt) * L->dalp[c00] + dt * L->dalp[c01];
        *lw = (1.0 - dt) * m->lw[c00] + dt * m->lw[c01];
        *nup = (1.0 - dt) * NU(c00) + dt * NU(c01);
        *ndn = (1.0 - dt) * ND(c00) + dt * ND(c01);
        for (int i = 0; i < 3; i++) v[i] = (1.0 - dt) * m->vel[3 * c00 + i] + dt * m->vel[3 * c01 + i];
    } else if (icr == 2) {
        *srcd = (1.0 - dr) * L->dsrc[c00] + dr * L->dsrc[c10];
        *alpd = (1.0 - dr) * L->dalp[c00] + dr * L->dalp[c10];
        *lw = (1.0 - dr) * m->lw[c00] + dr * m->lw[c10];
        *nup = (1.0 - dr) * NU(c00) + dr * NU(c10);
        *ndn = (1.0 - dr) * ND(c00) + dr * ND(c10);
        for (int i = 0; i < 3; i++) v[i] = (1.0 - dr) * m->vel[3 * c00 + i] + dr * m->vel[3 * c10 + i];
    } else {
#define BIL(f) ((1.0 - dr) * ((1.0 - dt) * (f(c00)) + dt * (f(c01))) + dr * ((1.0 - dt) * (f(c10)) + dt * (f(c11))))
#define FS(c) L->dsrc[c]
#define FA(c) L->dalp[c]
#define FW(c) m->lw[c]
        *srcd = BIL(FS); *alpd = BIL(FA); *lw = BIL(FW); *nup = BIL(NU); *ndn = BIL(ND);
        for (int i = 0; i < 3; i++) {
#define FV(c) m->vel[3 * (c) + i]
            v[i] = BIL(FV);
#undef FV
        }
#undef BIL
#undef FS
#undef FA
#undef FW
    }
#undef NU
#undef ND
    if (mu > 1.0) return fail("node: mu > 1");
    *dvmu = 3.335668e-11 * (mu * v[0] + sqrt(1.0 - mu * mu) * (v[1] * sin(phi) + v[2] * cos(phi)));
    return 0;
}

static double voigt(double nu00, double aks, double dnu) {
    double nu0 = fabs(nu00);
    double aa = 3.33567e-6 * nu0 * aks;
    double norm = 0.56419583546 / aa;
    double u = dnu / aa;
    return norm * exp(-(u * u));
}

/* The overshoot test (transfer.F:1548-1553, on in the reference's default build): the
   quadrature before the bracket above twice the theoretical maximum; counted, then bracketed
   as usual. */
static double qdr_src_2(double in, double js1, double alp1, double js2, double alp2, double ds, long long* nover) {
    double dtau1 = 0.5 * (alp1 + alp2) * ds;
    double theomax = 0.5 * (js1 + js2) * ds;
    double xp, a, b;
    if (dtau1 > 1.0e-6) { xp = exp(-dtau1); double e0 = 1.0 - xp; double e1 = dtau1 - e0; b = e1 / dtau1; a = e0 - b; }
    else { a = 0.5 * dtau1; b = 0.5 * dtau1; xp = 1.0 - dtau1; }
    double src1, src2, q;
    if (alp1 > 0.0) src1 = js1 / alp1; else if (alp2 > 0.0) src1 = js2 / alp2; else src1 = 0.0;
    if (alp2 > 0.0) src2 = js2 / alp2; else if (alp1 > 0.0) src2 = js1 / alp1; else src2 = 0.0;
    if (dtau1 > (double)1e-9f) q = a * src1 + b * src2; else q = 0.5 * (js1 + js2) * ds;
    if (q > 2.0 * theomax) (*nover)++;
    if (q > theomax) q = theomax;
    return in * xp + q;
}

typedef struct { double phiprof0, srcl0, alpl0; int init; } lstate;

static void integrate_el(linectx* L, int inu, double* I, double ds, double sd0, double sd1, double ad0, double ad1,
                         double lw0, double lw1, double dv0, double dv1, double nu0, double nu1, double nd0, double nd1,
                         lstate* st) {
    double lwav = 0.5 * (lw0 + lw1);
    double dn0 = L->dnu[inu] - L->lfreq * dv0;
    double dn1 = L->dnu[inu] - L->lfreq * dv1;
    if (st->init == 1) st->phiprof0 = voigt(L->lfreq, lwav, dn0);
    double phi1 = voigt(L->lfreq, lwav, dn1);
    if (st->init == 1) st->srcl0 = 5.27296241956e-28 * L->lfreq * nu0 * L->Aud * st->phiprof0;
    double srcl1 = 5.27296241956e-28 * L->lfreq * nu1 * L->Aud * phi1;
    if (st->init == 1) st->alpl0 = 5.27296241956e-28 * L->lfreq * st->phiprof0 * (nd0 * L->Bdu - nu0 * L->Bud);
    double alpl1 = 5.27296241956e-28 * L->lfreq * phi1 * (nd1 * L->Bdu - nu1 * L->Bud);
    double src0 = sd0 + st->srcl0, src1 = sd1 + srcl1, alp0 = ad0 + st->alpl0, alp1 = ad1 + alpl1;
    *I = qdr_src_2(*I, src0, alp0, src1, alp1, ds, &L->overshoot);
    L->tau = L->tau + 0.5 * (alp0 + alp1) * ds;
    st->phiprof0 = phi1; st->srcl0 = srcl1; st->alpl0 = alpl1; st->init = 0;
    L->steps++;
}

static void clever_integrate(linectx* L, int inu, double* I, double ds, double sd0, double sd1, double ad0, double ad1,
                             double lw0, double lw1, double dv0, double dv1, double nu0, double nu1, double nd0, double nd1,
                             lstate* st) {
    double lw = 0.5 * (lw0 + lw1);
    double q = fabs((dv1 - dv0) / (lw / 2.99792458e5));
    if (2.0 * 3.0 * q > 1.0) {
        double s_c = ds * ((L->dnu[inu] / L->lfreq) - dv0) / (dv1 - dv0);
        double dls = ds / q;
        double sright = s_c + 3.0 * dls, sleft = s_c - 3.0 * dls;
        if (sright > 0.0 && sleft < ds) {
            const int nmax = 31;
            double lg_s[34], lnu[34], lnd[34], ldv[34], lsd[34], lad[34];
            double lg_ds = (sright - sleft) / (nmax - 1.0);
            int n = 1;
            lg_s[1] = 0.0; lnu[1] = nu0; lnd[1] = nd0; ldv[1] = dv0; lsd[1] = sd0; lad[1] = ad0;
            for (int i = 1; i <= nmax; i++) {
                double s = sleft + (i - 1) * lg_ds;
                if (s > 0.0 && s < ds) {
                    double e = s / ds, ep = 1.0 - e;
                    n++;
                    lg_s[n] = s; lnu[n] = ep * nu0 + e * nu1; lnd[n] = ep * nd0 + e * nd1;
                    ldv[n] = ep * dv0 + e * dv1; lsd[n] = ep * sd0 + e * sd1; lad[n] = ep * ad0 + e * ad1;
                }
            }
            n++;
            lg_s[n] = ds; lnu[n] = nu1; lnd[n] = nd1; ldv[n] = dv1; lsd[n] = sd1; lad[n] = ad1;
            for (int i = 2; i <= n; i++)
                integrate_el(L, inu, I, lg_s[i] - lg_s[i - 1], lsd[i - 1], lsd[i], lad[i - 1], lad[i], lw, lw,
                             ldv[i - 1], ldv[i], lnu[i - 1], lnu[i], lnd[i - 1], lnd[i], st);
            return;
        }
    }
    integrate_el(L, inu, I, ds, sd0, sd1, ad0, ad1, lw0, lw1, dv0, dv1, nu0, nu1, nd0, nd1, st);
}

/* one (ray, channel): charintline (telescope.F:3889-4312) */
static int charint(linectx* L, const traj_t* T, int inu, double rbeam0, float* minvel, float* maxvel, double* out) {
    const rlo_model* m = L->m;
    double I = 0.0; int istar_done = 0;
    lstate st = {0, 0, 0, 1};
    int icr = T->icr[1], ir = T->ir[1], it = T->it[1];
    double r = T->r[1], th = T->th[1];
    double dr = (r - RG(m, ir)) / (RG(m, ir + 1) - RG(m, ir));
    double dt = (th - TG(m, it)) / (TG(m, it + 1) - TG(m, it));
    double sd0 = 0, ad0 = 0, lw0 = 0, dv0 = 0, nu0 = 0, nd0 = 0;
    if (ir == 0) I = L->star[inu];
    else {
        if (m->outer_bc == 2) {
            double fq = L->lfreq, temp = 2.728;
            I = 1.47455253991e-47 * (fq * fq * fq) / (exp(4.7991598e-11 * fq / temp) - 1.0);
        } else if (m->outer_bc == 3) {
            I = L->isrf ? L->isrf[inu] : 0.0;   /* radbnd_interstellfield(inu), telescope.F:4016-4023 */
        } else I = 0.0;
        if (node_values(L, icr, ir, it, dr, dt, T->mu[1], T->phi[1], &sd0, &ad0, &dv0, &lw0, &nu0, &nd0)) return -1;
    }
    for (int is = 2; is <= T->n; is++) {
        double ds = T->s[is] - T->s[is - 1];
        if (ds < 0.0) return fail("walk: negative ds");
        int ir_old = ir, icr_old = icr;
        icr = T->icr[is]; r = T->r[is]; th = T->th[is]; ir = T->ir[is]; it = T->it[is];
        if (ir == 0) return fail("walk: stellar surface reached");
        dr = (r - RG(m, ir)) / (RG(m, ir + 1) - RG(m, ir));
        dt = (th - TG(m, it)) / (TG(m, it + 1) - TG(m, it));
        if (ir == 1 && ir_old == 1 && icr == 1 && icr_old == 1) { ds = 0.0; st.init = 1; }
        if (ir == 1 && ir_old == 0 && icr == 1 && icr_old == 1) { ds = 0.0; st.init = 1; }
        if (ir <= 1) {   /* inner boundary: vacuum with central star (type 2) */
            if (ir == 1 && istar_done == 0 && rbeam0 > 0.0) {
                if (rbeam0 < m->rstar) return fail("walk: central beam smaller than the star");
                double f = (m->rstar / rbeam0) * (m->rstar / rbeam0);
                I = (1.0 - f) * I + f * L->star[inu];
                istar_done = 1; st.init = 1;
            }
        }
        double sd1, ad1, lw1, dv1, nu1, nd1;
        if (node_values(L, icr, ir, it, dr, dt, T->mu[is], T->phi[is], &sd1, &ad1, &dv1, &lw1, &nu1, &nd1)) return -1;
        clever_integrate(L, inu, &I, ds, sd0, sd1, ad0, ad1, lw0, lw1, dv0, dv1, nu0, nu1, nd0, nd1, &st);
        if (st.alpl0 * ds < -0.01) L->maser = 1;   /* masing check, telescope.F:4291-4297 */
        if (dv0 < (double)*minvel && nu0 + nd0 > LEVTHRES) *minvel = (float)dv0;
        if (dv0 > (double)*maxvel && nu0 + nd0 > LEVTHRES) *maxvel = (float)dv0;
        sd0 = sd1; ad0 = ad1; lw0 = lw1; dv0 = dv1; nu0 = nu1; nd0 = nd1;
    }
    *out = I;
    return 0;
}

/* with_isrf: fill the interstellar start table as calc_line_spectrum does
   (line_init_passband_outerbc, line.F:3855-3903, called at telescope.F:1564-1570); the
   position-velocity path (calc_write_line_posvel, telescope.F:1828-1924) never fills it, so
   its rays start from the zeros of the untouched table. */
static int line_ctx(rlo_model* m, int il, linectx* L, int with_isrf) {
    memset(L, 0, sizeof *L);
    L->m = m; L->il = il;
    L->lfreq = m->lfreq[il]; L->nu0abs = fabs(L->lfreq); L->Aud = m->Aud[il];
    L->Bud = 6.78171833781e46 * L->Aud / (L->lfreq * L->lfreq * L->lfreq);
    L->Bdu = L->Bud * (m->g[m->lup[il]] / m->g[m->ldn[il]]);
    L->molpg = 1.0 / (m->umass * 1.6726e-24);
    int ncell = m->nr * m->nth;
    L->dsrc = &m->ldsrc[(size_t)il * ncell]; L->dalp = &m->ldalp[(size_t)il * ncell];
    int nfr = m->nfr;
    L->dnu = (double*)calloc((size_t)nfr + 1, sizeof(double));
    L->star = (double*)calloc((size_t)nfr + 1, sizeof(double));
    double passb = 3.33567e-6 * L->nu0abs * m->vmax, nu1 = 0.0 - passb, dnu = 2.0 * passb / (nfr - 1.0);
    for (int k = 1; k <= nfr; k++) {
        L->dnu[k] = nu1 + (k - 1) * dnu;
        double fq = L->nu0abs + L->dnu[k];
        int i = hunt1(m->cnu, m->ncont, fq, 0);
        if (i == 0 || i == m->ncont) L->star[k] = 0.0;
        else { double w = (fq - m->cnu[i]) / (m->cnu[i + 1] - m->cnu[i]); L->star[k] = (1.0 - w) * m->starcont[i] + w * m->starcont[i + 1]; }
    }
    if (with_isrf && m->outer_bc == 3) {
        L->isrf = (double*)calloc((size_t)nfr + 1, sizeof(double));
        for (int k = 1; k <= nfr; k++) {
            double fq = L->nu0abs + L->dnu[k];
            int i = hunt1(m->cnu, m->ncont, fq, 0);
            /* the zero test is against the channel count freq_nr, not the frequency count */
            if (i == 0 || i == nfr) L->isrf[k] = 0.0;
            else if (i >= m->ncont) {
                free(L->dnu); free(L->star); free(L->isrf);
                L->dnu = L->star = L->isrf = NULL;
                return fail("line %d channel %d: above the last frequency of frequency.inp (the reference reads past "
                            "interstellfield.inp there)", il, k);
            } else {
                double w = (fq - m->cnu[i]) / (m->cnu[i + 1] - m->cnu[i]);
                L->isrf[k] = (1.0 - w) * m->isrf[i] + w * m->isrf[i + 1];
            }
        }
    }
    return 0;
}

/* ----------------------------------------------------------------------------------- */
/* public entry points                                                                   */
/* ----------------------------------------------------------------------------------- */
int rlo_load_dir(const char* dir, rlo_model** out) {
    rlo_model* m = (rlo_model*)calloc(1, sizeof(rlo_model));
    if (read_model(dir, m) || setup_rays(m)) { rlo_free(m); *out = NULL; return -1; }
    prepare_line_dust(m);
    *out = m; return 0;
}

/* command and rectangular-image request of linespectrum.inp: iv = command, nx, ny, addstar;
   dv = szx, szy, phioff, xoff, yoff */
int rlo_pv_request(const rlo_model* m, int* iv, double* dv) {
    iv[0] = m->command; iv[1] = m->pv_nx; iv[2] = m->pv_ny; iv[3] = m->pv_addstar;
    dv[0] = m->pv_szx; dv[1] = m->pv_szy; dv[2] = m->pv_phioff; dv[3] = m->pv_xoff; dv[4] = m->pv_yoff;
    return 0;
}

int rlo_info(const rlo_model* m, int* info, double* dinfo) {
    info[0] = m->nr; info[1] = m->nth; info[2] = m->nlspec; info[3] = m->ilstart; info[4] = m->nfr;
    info[5] = m->nrays; info[6] = m->nphi; info[7] = m->nrr; info[8] = m->nlin; info[9] = m->nlev;
    dinfo[0] = m->incl_rad; dinfo[1] = m->vmax; dinfo[2] = m->rstar; dinfo[3] = m->aksmax; dinfo[4] = m->theta0;
    return 0;
}

int rlo_rays(const rlo_model* m, double* x0, double* z0, double* rays_r, double* ri) {
    for (int i = 0; i < m->nrays; i++) { x0[i] = m->x0[i + 1]; z0[i] = m->z0[i + 1]; }
    for (int i = 0; i <= m->nrr; i++) rays_r[i] = m->rays_r[i];
    for (int i = 0; i <= m->nrr + 1; i++) ri[i] = m->ri[i];
    return 0;
}

int rlo_trajectory(const rlo_model* m, int iray, int maxn, double* s, double* r, double* th, double* mu,
                   double* phi, int* icr, int* ir, int* it) {
    traj_t T; memset(&T, 0, sizeof T);
    if (iray < 0 || iray >= m->nrays) return fail("ray index out of range");
    if (trajectory(m, m->x0[iray + 1], m->z0[iray + 1], m->theta0, &T)) { traj_free(&T); return -1; }
    int n = T.n < maxn ? T.n : maxn;
    for (int k = 0; k < n; k++) {
        s[k] = T.s[k + 1]; r[k] = T.r[k + 1]; th[k] = T.th[k + 1]; mu[k] = T.mu[k + 1]; phi[k] = T.phi[k + 1];
        icr[k] = T.icr[k + 1]; ir[k] = T.ir[k + 1]; it[k] = T.it[k + 1];
    }
    int tot = T.n; traj_free(&T);
    return tot;
}

/* The image of one line over rays [ray_begin, ray_end): image[(ray-ray_begin)*nfr + k],
   mask = imcir_cmask of this line alone (telescope.F:548,575): 1 for channel 1 and the
   channels inside the ray's velocity window, 0 for continuum copies and for the channel
   that computes a missing continuum; all 1 on the central beam, whose mask the reference
   never writes. counts[0] = formal-solution steps, counts[1] = integrated (ray, channel)
   pairs, counts[2] = nodes walked. */
int rlo_line_image(rlo_model* m, int iline, int ray_begin, int ray_end, double* image, unsigned char* mask,
                   long long* counts) {
    if (iline < 1 || iline > m->nlin) return fail("line index out of range");
    if (ray_begin < 0 || ray_end > m->nrays || ray_begin > ray_end) return fail("ray range out of bounds");
    linectx L; if (line_ctx(m, iline, &L, 1)) return -1;
    int nfr = m->nfr; int rc = 0;
    double* velo = (double*)malloc(sizeof(double) * (nfr + 1));
    for (int k = 1; k <= nfr; k++) velo[k] = L.dnu[k] / L.lfreq;
    double aksmax_c = m->aksmax / 2.99792458e5;
    long long integ = 0, nodes = 0;
    for (int ray = ray_begin; ray < ray_end && !rc; ray++) {
        traj_t T; memset(&T, 0, sizeof T);
        if (trajectory(m, m->x0[ray + 1], m->z0[ray + 1], m->theta0, &T)) { traj_free(&T); rc = -1; break; }
        double* img = &image[(size_t)(ray - ray_begin) * nfr];
        unsigned char* msk = mask ? &mask[(size_t)(ray - ray_begin) * nfr] : NULL;
        float minv = 1.0f, maxv = -1.0f;
        if (ray == 0) {
            for (int k = 1; k <= nfr && !rc; k++) {
                rc = charint(&L, &T, k, m->ri[1], &minv, &maxv, &img[k - 1]);
                if (msk) msk[k - 1] = 1;
                integ++; nodes += T.n;
            }
        } else {
            double cont = 0.0;
            rc = charint(&L, &T, 1, -1.0, &minv, &maxv, &img[0]);
            if (msk) msk[0] = 1;
            integ++; nodes += T.n;
            if (velo[1] > maxv + 2.0 * aksmax_c || velo[1] < minv - 2.0 * aksmax_c) cont = img[0];
            for (int k = 2; k <= nfr && !rc; k++) {
                if (velo[k] <= maxv + 2.0 * aksmax_c && velo[k] >= minv - 2.0 * aksmax_c) {
                    rc = charint(&L, &T, k, -1.0, &minv, &maxv, &img[k - 1]);
                    if (msk) msk[k - 1] = 1;
                    integ++; nodes += T.n;
                } else if (cont != 0.0) {
                    img[k - 1] = cont;
                    if (msk) msk[k - 1] = 0;
                } else {
                    rc = charint(&L, &T, k, -1.0, &minv, &maxv, &img[k - 1]);
                    cont = img[k - 1];
                    if (msk) msk[k - 1] = 0;
                    integ++; nodes += T.n;
                }
            }
        }
        traj_free(&T);
    }
    if (counts) { counts[0] = L.steps; counts[1] = integ; counts[2] = nodes; }
    m->maser = L.maser;
    m->overshoot = L.overshoot;
    free(velo); free(L.dnu); free(L.star); free(L.isrf);
    return rc;
}

/* Every channel of one ray (x0, z0) at the camera's inclination, without the NONREDUNDANT
   window and without central-star mixing: one pixel of the rectangular image
   (make_freq_image_rectang, telescope.F:2061-2150; charintline with rbeam 0). I and the
   line-of-sight optical depth char_tau per channel. With outer boundary 3 the rays start
   at 0: the position-velocity path leaves the interstellar table unfilled. */
int rlo_ray_spectrum(rlo_model* m, int iline, double x0, double z0, double* I_out, double* tau_out) {
    if (iline < 1 || iline > m->nlin) return fail("line index out of range");
    linectx L; if (line_ctx(m, iline, &L, 0)) return -1;
    traj_t T; memset(&T, 0, sizeof T);
    int rc = trajectory(m, x0, z0, m->theta0, &T);
    for (int k = 1; k <= m->nfr && !rc; k++) {
        float minv = 1.0f, maxv = -1.0f;
        L.tau = 0.0;
        rc = charint(&L, &T, k, 0.0, &minv, &maxv, &I_out[k - 1]);
        if (tau_out) tau_out[k - 1] = L.tau;
    }
    m->maser |= L.maser;
    m->overshoot += L.overshoot;
    traj_free(&T);
    free(L.dnu); free(L.star);
    return rc;
}

/* Rectangular camera (setup_rays_rectang, telescope.F:2229-2475) of the request
   (nx, ny, szx, szy, phioff, xoff, yoff, addstar): pixel rays in the reference's order
   (ix outer, iy inner), x0/z0/b of [nx*ny]. info[0] = 1 when the unresolved star is added;
   dinfo: spx, spy, srat, theta0. */
int rlo_pv_rays(const rlo_model* m, int nx, int ny, double szx, double szy, double phioff, double xoff, double yoff,
                int addstar, double* x0, double* z0, double* b, int* info, double* dinfo) {
    if (nx < 2 || ny < 2 || nx % 2 || ny % 2) return fail("rectangular image: nx, ny must be even");
    double spx = (szx * 0.5) / (nx * 0.5), spy = (szy * 0.5) / (ny * 0.5);
    if (!(spx > 0.0) || !(spy > 0.0)) return fail("rectangular image: pixel size must be positive");
    if (addstar > 0 && (xoff != 0.0 || yoff != 0.0)) return fail("rectangular image: star needs zero offsets");
    double anginf = m->incl_rad;
    if (anginf < 1.0e-1) anginf = (double)0.1f;
    double theta0 = anginf + 1.0e-4, sinth0 = sin(theta0);
    int ir = 0;
    for (int ix = 1; ix <= nx; ix++) {
        for (int iy = 1; iy <= ny; iy++) {
            double x_c = (ix - nx / 2 - 0.5) * spx - xoff;
            double y_c = (iy - ny / 2 - 0.5) * spy - yoff;
            double r_c = sqrt(x_c * x_c + y_c * y_c);
            if (x_c == 0.0) x_c = x_c + 0.001 * spx;
            double p_c = atan(y_c / x_c) - phioff;
            if (x_c < 0.0) p_c = p_c + 3.14159265359;
            while (p_c < 0.0) p_c = p_c + 6.28318530718;
            while (p_c >= 6.28318530718) p_c = p_c - 6.28318530718;
            double zh0 = -sin(p_c) / sinth0;
            double dum = 1.0 - zh0 * zh0 * sinth0 * sinth0 + 1e-4;
            double xh0 = cos(p_c) > 0.0 ? sqrt(dum) : -sqrt(dum);
            x0[ir] = r_c * xh0; z0[ir] = r_c * zh0; b[ir] = r_c;
            ir++;
        }
    }
    info[0] = addstar > 0 && spx * spx + spy * spy > m->rstar * m->rstar;
    dinfo[0] = spx; dinfo[1] = spy;
    dinfo[2] = (3.14159265 * (m->rstar * m->rstar)) / (4.0 * spx * spy);
    dinfo[3] = theta0;
    return 0;
}

/* The position-velocity cube of one line (make_freq_image_rectang, telescope.F:2061-2206):
   I and tau of [nfr][ny][nx] (per channel, iy outer, ix inner). */
int rlo_posvel(rlo_model* m, int iline, int nx, int ny, double szx, double szy, double phioff, double xoff,
               double yoff, int addstar, double* I, double* tau) {
    if (iline < 1 || iline > m->nlin) return fail("line index out of range");
    int npix = nx * ny, info[1]; double dinfo[4];
    double* x0 = (double*)malloc(sizeof(double) * (size_t)npix * 3);
    if (!x0) return fail("out of memory");
    double *z0 = x0 + npix, *b = z0 + npix;
    int rc = rlo_pv_rays(m, nx, ny, szx, szy, phioff, xoff, yoff, addstar, x0, z0, b, info, dinfo);
    m->maser = 0;
    m->overshoot = 0;
    double theta_saved = m->theta0;
    m->theta0 = dinfo[3];
    double rmax = RG(m, m->nr);
    int nfr = m->nfr;
    double *Ir = (double*)malloc(sizeof(double) * nfr * 2), *tr = Ir + nfr;
    for (int ix = 1; ix <= nx && !rc; ix++) {
        for (int iy = 1; iy <= ny && !rc; iy++) {
            int r = (ix - 1) * ny + (iy - 1);
            if (b[r] < 0.999 * rmax) rc = rlo_ray_spectrum(m, iline, x0[r], z0[r], Ir, tr);
            else for (int k = 0; k < nfr; k++) { Ir[k] = 0.0; tr[k] = 0.0; }
            for (int k = 0; k < nfr; k++) {
                size_t o = ((size_t)k * ny + (iy - 1)) * nx + (ix - 1);
                I[o] = Ir[k]; tau[o] = tr[k];
            }
        }
    }
    if (!rc && info[0]) {   /* the unresolved star over the four central pixels */
        double srat = dinfo[2], srat1 = 1.0 - srat;
        rc = rlo_ray_spectrum(m, iline, 0.0, 0.0, Ir, tr);
        for (int k = 0; k < nfr && !rc; k++) {
            double dummy = Ir[k] * srat;
            for (int dx = 0; dx < 2; dx++)
                for (int dy = 0; dy < 2; dy++) {
                    size_t o = ((size_t)k * ny + (ny / 2 - 1 + dy)) * nx + (nx / 2 - 1 + dx);
                    I[o] = dummy + srat1 * I[o];
                }
        }
    }
    m->theta0 = theta_saved;
    free(Ir); free(x0);
    return rc;
}

/* image -> F_nu at 1 pc (telescope.F:1320-1437). image covers all rays. */
int rlo_image_to_spectrum(const rlo_model* m, const double* image, double* flux) {
    int nfr = m->nfr, nphi = m->nphi;
    double dist = 1.0 * 3.08572e18;
    for (int k = 0; k < nfr; k++) {
        double slum = 0.0;
        double surf = 3.14159265359 * (m->ri[1] * m->ri[1]);
        slum = slum + surf * image[k];
        for (int ir = 1; ir <= m->nrr; ir++) {
            surf = 3.14159265359 * (m->ri[ir + 1] * m->ri[ir + 1] - m->ri[ir] * m->ri[ir]);
            double d = 0.0;
            for (int ip = 0; ip < nphi; ip++) d = d + image[(size_t)(1 + (ir - 1) * nphi + ip) * nfr + k];
            d = d / (1.0 * nphi);
            d = d * surf;
            slum = slum + d;
        }
        flux[k] = slum / (dist * dist);
    }
    return 0;
}

int rlo_masing(const rlo_model* m) { return m->maser; }
long long rlo_overshoots(const rlo_model* m) { return m->overshoot; }

int rlo_line_spectrum(rlo_model* m, int iline, double* flux, double* velo_kms, long long* counts) {
    size_t n = (size_t)m->nrays * m->nfr;
    double* img = (double*)malloc(sizeof(double) * n);
    if (!img) return fail("out of memory");
    int rc = rlo_line_image(m, iline, 0, m->nrays, img, NULL, counts);
    if (!rc) rc = rlo_image_to_spectrum(m, img, flux);
    if (!rc && velo_kms) {
        double lf = m->lfreq[iline], nu0 = fabs(lf);
        double passb = 3.33567e-6 * nu0 * m->vmax, dnu = 2.0 * passb / (m->nfr - 1.0);
        for (int k = 0; k < m->nfr; k++) {
            double fq = nu0 + (-passb + k * dnu);
            velo_kms[k] = -2.99792458e5 * (fq - lf) / lf + m->radvelo;
        }
    }
    free(img);
    return rc;
}

/* gfortran-style Ew.d edit descriptor */
static void fmt_E(char* out, double v, int w, int d) {
    char tmp[64], body[64];
    int neg = v < 0 || (v == 0 && signbit(v));
    double a = fabs(v); int ex = 0; char dig[40];
    if (a == 0.0) { memset(dig, '0', (size_t)d); dig[d] = 0; ex = 0; }
    else {
        snprintf(tmp, sizeof tmp, "%.*e", d - 1, a);
        int k = 0; for (char* p = tmp; *p && *p != 'e'; p++) if (isdigit((unsigned char)*p)) dig[k++] = *p;
        dig[k] = 0; ex = atoi(strchr(tmp, 'e') + 1) + 1;
    }
    char expo[16];
    if (abs(ex) <= 99) snprintf(expo, sizeof expo, "E%c%02d", ex < 0 ? '-' : '+', abs(ex));
    else snprintf(expo, sizeof expo, "%c%03d", ex < 0 ? '-' : '+', abs(ex));
    int need0 = (d + 6 + neg) <= w;
    snprintf(body, sizeof body, "%s%s.%s%s", neg ? "-" : "", need0 ? "0" : "", dig, expo);
    int L = (int)strlen(body);
    if (L > w) { memset(out, '*', (size_t)w); out[w] = 0; return; }
    snprintf(out, (size_t)w + 1, "%*s", w, body);
}

/* Whole run in a directory, like the RADlite executable: linespectrum_<mol>.dat and
   radlite.success. Returns 0 on success. */
int rlo_run_dir(const char* dir) {
    rlo_model* m;
    if (rlo_load_dir(dir, &m)) return -1;
    if (m->style != 1) { rlo_free(m); return fail("only output style 1 (F_nu) is supported without a beam"); }
    if (m->command != 0) { rlo_free(m); return fail("the oracle's run writes line spectra (command 0) only"); }
    char path[1024]; snprintf(path, sizeof path, "%s/linespectrum_%s.dat", dir, m->molname);
    FILE* fp = fopen(path, "w");
    if (!fp) { rlo_free(m); return fail("cannot write %s", path); }
    char e1[32], e2[32];
    char fname[260]; snprintf(fname, sizeof fname, "./%s", m->molfile);
    fprintf(fp, "%2d\n%2d\n%-80s\n%-80s\n%10d\n%10d\n", 1, m->style, m->molname, fname, m->nlspec, m->nfr);
    fmt_E(e1, 1.0, 12, 4); fmt_E(e2, m->radvelo, 12, 4);
    fprintf(fp, "%s%s%7.3f\n", e1, e2, m->incl_rad * 57.2957795132);
    int rc = 0;
    double* flux = (double*)malloc(sizeof(double) * m->nfr);
    double* velo = (double*)malloc(sizeof(double) * m->nfr);
    for (int il = m->ilstart; il < m->ilstart + m->nlspec && !rc; il++) {
        rc = rlo_line_spectrum(m, il, flux, velo, NULL);
        if (rc) break;
        char ef[32], eb[32]; fmt_E(ef, m->lfreq[il], 14, 9); fmt_E(eb, 0.0, 10, 5);
        fprintf(fp, "\n%5d%5d\n%s\n%s\n%5d\n  \n", m->lup[il], m->ldn[il], ef, eb, m->nfr);
        for (int k = m->nfr - 1; k >= 0; k--) { fmt_E(e1, velo[k], 13, 6); fmt_E(e2, flux[k], 13, 6); fprintf(fp, "%s %s\n", e1, e2); }
    }
    fclose(fp); free(flux); free(velo); rlo_free(m);
    if (rc) return -1;
    snprintf(path, sizeof path, "%s/radlite.success", dir);
    fp = fopen(path, "w"); if (fp) { fprintf(fp, " 1\n"); fclose(fp); }
    return 0;
}

#ifdef RLO_MAIN
int main(int argc, char** argv) {
    const char* dir = argc > 1 ? argv[1] : ".";
    if (rlo_run_dir(dir)) { fprintf(stderr, "rl_oracle: %s\n", rlo_last_error()); return 13; }
    return 0;
}
#endif
