/*
 * workloads.c -- seeded synthetic LDU workloads (inputs only).
 *
 * Generates the benchmark and test systems: structured 5/7-point grids in
 * OpenFOAM upper-triangular face order with constant, lognormal(0,1), upwind
 * convection-diffusion or Gaussian-random-field diffusion coefficients, plus
 * uniform sources and random permutations.  Only correctly rounded IEEE
 * operations are used (elementary functions are evaluated from range
 * reduction and Taylor series here, not from libm) and the file is compiled
 * with -ffp-contract=off, so every host produces the same bytes for the same
 * seed.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================= */
/* deterministic random numbers                                            */
/* ======================================================================= */

uint64_t wl_splitmix64(uint64_t *state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double wl_uniform01(uint64_t *state)
{
    return (double)(wl_splitmix64(state) >> 11) * (1.0 / 9007199254740992.0);
}

/* Elementary functions from range reduction + Taylor series using only
 * correctly rounded IEEE operations, so generated inputs are bit-identical
 * on every host.  Accuracy is ~1e-15 relative, which is all the generators
 * need. */
static const double K_LN2 = 0.6931471805599453094172321;
static const double K_LN2_LO = 2.319046813846299558e-17;
static const double K_2PI = 6.283185307179586476925287;
static const double K_2PI_LO = 2.4492935982947064e-16;

double wl_exp(double x)
{
    if (x != x) return x;
    if (x > 709.0) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    double kd = nearbyint(x / K_LN2);
    double r = (x - kd * K_LN2) - kd * K_LN2_LO;
    double p = 1.0;
    for (int i = 18; i >= 1; --i) p = 1.0 + (r * p) / (double)i;
    return ldexp(p, (int)kd);
}

double wl_log(double x)
{
    if (!(x > 0.0)) return (x == 0.0) ? -HUGE_VAL : NAN;
    if (x == HUGE_VAL) return x;
    int e;
    double m = frexp(x, &e); /* m in [0.5, 1) */
    if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double sum = 0.0;
    for (int i = 16; i >= 0; --i) sum = 1.0 / (double)(2 * i + 1) + s2 * sum;
    double lm = 2.0 * s * sum;
    return ((double)e * K_LN2 + lm) + (double)e * K_LN2_LO;
}

static double reduce_2pi(double x)
{
    double k = nearbyint(x / K_2PI);
    return (x - k * K_2PI) - k * K_2PI_LO;
}

double wl_sin(double x)
{
    double r = reduce_2pi(x);
    double r2 = r * r;
    double p = 0.0;
    /* sum_{i>=0} (-1)^i r^(2i+1)/(2i+1)!  by Horner in r^2 */
    for (int i = 17; i >= 1; --i) p = 1.0 - (r2 * p) / (double)((2 * i) * (2 * i + 1));
    return r * p;
}

double wl_cos(double x)
{
    double r = reduce_2pi(x);
    double r2 = r * r;
    double p = 0.0;
    for (int i = 17; i >= 1; --i) p = 1.0 - (r2 * p) / (double)((2 * i - 1) * (2 * i));
    return p;
}

void wl_fill_uniform(uint64_t seed, double lo, double hi, double *out, int64_t n)
{
    uint64_t s = seed;
    double w = hi - lo;
    for (int64_t i = 0; i < n; ++i) out[i] = lo + w * wl_uniform01(&s);
}

/* Marsaglia polar method; both variates of each accepted pair are used. */
void wl_fill_normal(uint64_t seed, double *out, int64_t n)
{
    uint64_t s = seed;
    int64_t i = 0;
    while (i < n) {
        double u = 2.0 * wl_uniform01(&s) - 1.0;
        double v = 2.0 * wl_uniform01(&s) - 1.0;
        double q = u * u + v * v;
        if (q >= 1.0 || q == 0.0) continue;
        double f = sqrt(-2.0 * wl_log(q) / q);
        out[i++] = u * f;
        if (i < n) out[i++] = v * f;
    }
}

/* Fisher-Yates shuffle of 0..n-1. */
void wl_permutation(uint64_t seed, int32_t n, int32_t *perm)
{
    uint64_t s = seed;
    for (int32_t i = 0; i < n; ++i) perm[i] = i;
    for (int32_t i = n - 1; i > 0; --i) {
        int32_t j = (int32_t)(wl_splitmix64(&s) % (uint64_t)(i + 1));
        int32_t t = perm[i]; perm[i] = perm[j]; perm[j] = t;
    }
}

/* ======================================================================= */
/* structured grid generators                                              */
/* ======================================================================= */
/* Cells are numbered c = i + nx*(j + ny*k).  Faces are listed owner by
 * owner; the faces of owner c go to c+1, c+nx, c+nx*ny in that order, so
 * the face list is sorted by owner, then by neighbour: OpenFOAM's
 * upper-triangular order. */

int64_t wl_grid_n_faces(int32_t nx, int32_t ny, int32_t nz)
{
    return (int64_t)(nx - 1) * ny * nz + (int64_t)nx * (ny - 1) * nz +
           (int64_t)nx * ny * (nz - 1);
}

void wl_grid_addressing(int32_t nx, int32_t ny, int32_t nz,
                         int32_t *lower_addr, int32_t *upper_addr)
{
    int64_t f = 0;
    const int32_t sxy = nx * ny;
    for (int32_t k = 0; k < nz; ++k)
        for (int32_t j = 0; j < ny; ++j)
            for (int32_t i = 0; i < nx; ++i) {
                int32_t c = i + nx * (j + ny * k);
                if (i + 1 < nx) { lower_addr[f] = c; upper_addr[f] = c + 1; ++f; }
                if (j + 1 < ny) { lower_addr[f] = c; upper_addr[f] = c + nx; ++f; }
                if (k + 1 < nz) { lower_addr[f] = c; upper_addr[f] = c + sxy; ++f; }
            }
}

void wl_grid_const(int32_t nx, int32_t ny, int32_t nz, double diag_value,
                    double off_value, double *diag, double *lower, double *upper)
{
    int64_t n = (int64_t)nx * ny * nz, nf = wl_grid_n_faces(nx, ny, nz);
    for (int64_t c = 0; c < n; ++c) diag[c] = diag_value;
    for (int64_t f = 0; f < nf; ++f) { lower[f] = off_value; upper[f] = off_value; }
}

/* number of boundary faces of cell (i,j,k): directions without a neighbour */
static int n_boundary_faces(int32_t nx, int32_t ny, int32_t nz, int32_t i,
                            int32_t j, int32_t k)
{
    int b = (i == 0) + (i == nx - 1) + (j == 0) + (j == ny - 1);
    if (nz > 1) b += (k == 0) + (k == nz - 1);
    return b;
}

/* Face coefficients k ~ lognormal(0,1) (seeded); lower = upper = -k.
 * Every boundary face gets its own lognormal(0,1) coefficient folded into
 * the diagonal (Dirichlet), so diag_i = sum of |off-diagonals| + boundary
 * terms and A is symmetric positive definite. */
void wl_grid_lognormal(int32_t nx, int32_t ny, int32_t nz, uint64_t seed,
                        double *diag, double *lower, double *upper)
{
    int64_t n = (int64_t)nx * ny * nz, nf = wl_grid_n_faces(nx, ny, nz);
    int32_t *la = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nf > 0 ? nf : 1));
    int32_t *ua = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nf > 0 ? nf : 1));
    wl_grid_addressing(nx, ny, nz, la, ua);
    int64_t nb = 0;
    for (int32_t k = 0; k < nz; ++k)
        for (int32_t j = 0; j < ny; ++j)
            for (int32_t i = 0; i < nx; ++i) nb += n_boundary_faces(nx, ny, nz, i, j, k);
    double *z = (double *)malloc(sizeof(double) * (size_t)(nf + nb + 1));
    wl_fill_normal(seed, z, nf + nb);
    for (int64_t c = 0; c < n; ++c) diag[c] = 0.0;
    for (int64_t f = 0; f < nf; ++f) {
        double kf = wl_exp(z[f]);
        lower[f] = -kf;
        upper[f] = -kf;
        diag[la[f]] += kf;
        diag[ua[f]] += kf;
    }
    int64_t b = nf;
    for (int32_t k = 0; k < nz; ++k)
        for (int32_t j = 0; j < ny; ++j)
            for (int32_t i = 0; i < nx; ++i) {
                int64_t c = i + (int64_t)nx * (j + (int64_t)ny * k);
                int nbf = n_boundary_faces(nx, ny, nz, i, j, k);
                for (int q = 0; q < nbf; ++q) diag[c] += wl_exp(z[b++]);
            }
    free(z); free(la); free(ua);
}

/* ---- convection-diffusion (upwind) with a divergence-free velocity ----- */
/* The velocity is the discrete curl of a seeded smooth vector potential
 * psi (a sum of low-wavenumber Fourier modes per component).  Face fluxes
 * are circulations of psi around the face edges (midpoint rule), so the
 * discrete divergence of every cell vanishes up to rounding. */
#define CD_MODES 4
typedef struct {
    int32_t n[3];
    double amp[3][CD_MODES];
    /* tables over half-integer positions t/2, t = 0..2n */
    double *S[3][CD_MODES][3];
    double *C[3][CD_MODES][3];
} cd_potential;

static void cd_init(cd_potential *P, int32_t nx, int32_t ny, int32_t nz, uint64_t seed)
{
    uint64_t s = seed;
    P->n[0] = nx; P->n[1] = ny; P->n[2] = nz;
    for (int comp = 0; comp < 3; ++comp)
        for (int m = 0; m < CD_MODES; ++m) {
            P->amp[comp][m] = 2.0 * wl_uniform01(&s) - 1.0;
            double phase = K_2PI * wl_uniform01(&s);
            for (int ax = 0; ax < 3; ++ax) {
                int kw = 1 + (int)(wl_splitmix64(&s) % 3ULL);
                int32_t len = 2 * P->n[ax] + 1;
                double *S = (double *)malloc(sizeof(double) * (size_t)len);
                double *C = (double *)malloc(sizeof(double) * (size_t)len);
                for (int32_t t = 0; t < len; ++t) {
                    double arg = K_2PI * (double)kw * (0.5 * (double)t) / (double)P->n[ax];
                    if (ax == 0) arg += phase;
                    S[t] = wl_sin(arg);
                    C[t] = wl_cos(arg);
                }
                P->S[comp][m][ax] = S;
                P->C[comp][m][ax] = C;
            }
        }
}

static void cd_free(cd_potential *P)
{
    for (int comp = 0; comp < 3; ++comp)
        for (int m = 0; m < CD_MODES; ++m)
            for (int ax = 0; ax < 3; ++ax) { free(P->S[comp][m][ax]); free(P->C[comp][m][ax]); }
}

/* psi_comp at (tx/2, ty/2, tz/2): sum_m amp * sin(a + b + c) expanded by
 * angle addition over the per-axis tables. */
static double cd_psi(const cd_potential *P, int comp, int32_t tx, int32_t ty, int32_t tz)
{
    double acc = 0.0;
    for (int m = 0; m < CD_MODES; ++m) {
        double sa = P->S[comp][m][0][tx], ca = P->C[comp][m][0][tx];
        double sb = P->S[comp][m][1][ty], cb = P->C[comp][m][1][ty];
        double sc = P->S[comp][m][2][tz], cc = P->C[comp][m][2][tz];
        double sab = sa * cb + ca * sb;
        double cab = ca * cb - sa * sb;
        acc += P->amp[comp][m] * (sab * cc + cab * sc);
    }
    return acc;
}

/* Flux through the face with normal +axis located at integer coordinate
 * `pos` along axis, spanning [a, a+1] x [b, b+1] in the two other axes
 * (cyclic order).  Positions are passed as doubled integers. */
static double cd_flux(const cd_potential *P, int axis, int32_t x2, int32_t y2, int32_t z2)
{
    /* (x2,y2,z2): doubled coordinates of the face's low corner, with the
     * face-normal coordinate at the face plane. */
    if (axis == 0) { /* curl_x = d psi_z/dy - d psi_y/dz */
        return (cd_psi(P, 2, x2, y2 + 2, z2 + 1) - cd_psi(P, 2, x2, y2, z2 + 1)) -
               (cd_psi(P, 1, x2, y2 + 1, z2 + 2) - cd_psi(P, 1, x2, y2 + 1, z2));
    } else if (axis == 1) { /* curl_y = d psi_x/dz - d psi_z/dx */
        return (cd_psi(P, 0, x2 + 1, y2, z2 + 2) - cd_psi(P, 0, x2 + 1, y2, z2)) -
               (cd_psi(P, 2, x2 + 2, y2, z2 + 1) - cd_psi(P, 2, x2, y2, z2 + 1));
    } else { /* curl_z = d psi_y/dx - d psi_x/dy */
        return (cd_psi(P, 1, x2 + 2, y2 + 1, z2) - cd_psi(P, 1, x2, y2 + 1, z2)) -
               (cd_psi(P, 0, x2 + 1, y2 + 2, z2) - cd_psi(P, 0, x2 + 1, y2, z2));
    }
}

/* Upwind convection-diffusion, unit spacing, diffusivity 1 (face D = 1,
 * boundary D = 2 for the half-cell distance to a Dirichlet-0 wall).  For a
 * face with flux F from owner P to neighbour N:
 *   upper = A[P][N] = -(1 + max(-F,0)),  lower = A[N][P] = -(1 + max(F,0)),
 *   diag[P] += 1 + max(F,0),  diag[N] += 1 + max(-F,0).
 * Fluxes are scaled so that max |F| (the cell Peclet number) is pe_max.
 * pe_stats <- {min |F|, max |F|, fraction of faces with |F| < 0.1}. */
void wl_grid_convdiff(int32_t nx, int32_t ny, int32_t nz, uint64_t seed,
                       double pe_max, double *diag, double *lower, double *upper,
                       double *pe_stats)
{
    cd_potential P;
    cd_init(&P, nx, ny, nz, seed);
    const int64_t n = (int64_t)nx * ny * nz;
    const int64_t nf = wl_grid_n_faces(nx, ny, nz);
    /* face index of the first face of each owner: faces per cell depend only
     * on (i<nx-1, j<ny-1, k<nz-1); compute a prefix over cells */
    int64_t *fstart = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    fstart[0] = 0;
    for (int64_t c = 0; c < n; ++c) {
        int32_t i = (int32_t)(c % nx), j = (int32_t)((c / nx) % ny), k = (int32_t)(c / ((int64_t)nx * ny));
        fstart[c + 1] = fstart[c] + (i + 1 < nx) + (j + 1 < ny) + (k + 1 < nz);
    }
    double *flux = (double *)malloc(sizeof(double) * (size_t)(nf > 0 ? nf : 1));
    double maxabs = 0.0;
#pragma omp parallel for schedule(static) reduction(max : maxabs)
    for (int64_t c = 0; c < n; ++c) {
        int32_t i = (int32_t)(c % nx), j = (int32_t)((c / nx) % ny), k = (int32_t)(c / ((int64_t)nx * ny));
        int64_t f = fstart[c];
        if (i + 1 < nx) { flux[f] = cd_flux(&P, 0, 2 * (i + 1), 2 * j, 2 * k); if (fabs(flux[f]) > maxabs) maxabs = fabs(flux[f]); ++f; }
        if (j + 1 < ny) { flux[f] = cd_flux(&P, 1, 2 * i, 2 * (j + 1), 2 * k); if (fabs(flux[f]) > maxabs) maxabs = fabs(flux[f]); ++f; }
        if (k + 1 < nz) { flux[f] = cd_flux(&P, 2, 2 * i, 2 * j, 2 * (k + 1)); if (fabs(flux[f]) > maxabs) maxabs = fabs(flux[f]); ++f; }
    }
    double scale = (maxabs > 0.0) ? pe_max / maxabs : 0.0;
    double minabs = HUGE_VAL;
    int64_t nsmall = 0;
    for (int64_t f = 0; f < nf; ++f) {
        flux[f] *= scale;
        double a = fabs(flux[f]);
        if (a < minabs) minabs = a;
        if (a < 0.1) ++nsmall;
    }
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < n; ++c) diag[c] = 0.0;
    /* interior faces: owner-side and neighbour-side diagonal terms, applied
     * in face order (serial, so sums are order-deterministic) */
    for (int64_t c = 0; c < n; ++c) {
        int32_t i = (int32_t)(c % nx), j = (int32_t)((c / nx) % ny), k = (int32_t)(c / ((int64_t)nx * ny));
        int64_t f = fstart[c];
        int64_t nb[3] = {c + 1, c + nx, c + (int64_t)nx * ny};
        int has[3] = {i + 1 < nx, j + 1 < ny, k + 1 < nz};
        for (int d = 0; d < 3; ++d) {
            if (!has[d]) continue;
            double F = flux[f];
            double outP = F > 0.0 ? F : 0.0, outN = F < 0.0 ? -F : 0.0;
            upper[f] = -(1.0 + outN);
            lower[f] = -(1.0 + outP);
            diag[c] += 1.0 + outP;
            diag[nb[d]] += 1.0 + outN;
            ++f;
        }
    }
    /* boundary faces: outward flux through each wall face */
    for (int64_t c = 0; c < n; ++c) {
        int32_t i = (int32_t)(c % nx), j = (int32_t)((c / nx) % ny), k = (int32_t)(c / ((int64_t)nx * ny));
        double Fo;
        if (i == 0)      { Fo = -scale * cd_flux(&P, 0, 0, 2 * j, 2 * k);        diag[c] += 2.0 + (Fo > 0.0 ? Fo : 0.0); }
        if (i == nx - 1) { Fo = scale * cd_flux(&P, 0, 2 * nx, 2 * j, 2 * k);    diag[c] += 2.0 + (Fo > 0.0 ? Fo : 0.0); }
        if (j == 0)      { Fo = -scale * cd_flux(&P, 1, 2 * i, 0, 2 * k);        diag[c] += 2.0 + (Fo > 0.0 ? Fo : 0.0); }
        if (j == ny - 1) { Fo = scale * cd_flux(&P, 1, 2 * i, 2 * ny, 2 * k);    diag[c] += 2.0 + (Fo > 0.0 ? Fo : 0.0); }
        if (nz > 1) {
            if (k == 0)      { Fo = -scale * cd_flux(&P, 2, 2 * i, 2 * j, 0);     diag[c] += 2.0 + (Fo > 0.0 ? Fo : 0.0); }
            if (k == nz - 1) { Fo = scale * cd_flux(&P, 2, 2 * i, 2 * j, 2 * nz); diag[c] += 2.0 + (Fo > 0.0 ? Fo : 0.0); }
        }
    }
    if (pe_stats) {
        pe_stats[0] = nf > 0 ? minabs : 0.0;
        pe_stats[1] = nf > 0 ? maxabs * scale : 0.0;
        pe_stats[2] = nf > 0 ? (double)nsmall / (double)nf : 0.0;
    }
    free(flux); free(fstart);
    cd_free(&P);
}

/* ---- Gaussian random field (separable Gaussian filter of white noise) -- */
/* Covariance exp(-r^2 / (2 l^2)) with l = corr_len: white noise convolved
 * with a Gaussian kernel of standard deviation l/sqrt(2), normalised to
 * unit marginal variance.  Noise is drawn on a grid padded by the kernel
 * radius so the field has no boundary artefacts. */
void wl_grid_grf(int32_t nx, int32_t ny, int32_t nz, uint64_t seed,
                  double corr_len, double *g)
{
    double s = corr_len / sqrt(2.0);
    int32_t R = (int32_t)ceil(3.0 * s);
    int32_t W = 2 * R + 1;
    double *w = (double *)malloc(sizeof(double) * (size_t)W);
    double w2 = 0.0;
    for (int32_t t = -R; t <= R; ++t) {
        w[t + R] = wl_exp(-(double)(t * t) / (2.0 * s * s));
        w2 += w[t + R] * w[t + R];
    }
    int32_t px = nx + 2 * R, py = ny + 2 * R, pz = nz + 2 * R;
    int64_t np = (int64_t)px * py * pz;
    double *a = (double *)malloc(sizeof(double) * (size_t)np);
    wl_fill_normal(seed, a, np);
    /* convolve along x: a (px,py,pz) -> b (nx,py,pz) */
    double *b = (double *)malloc(sizeof(double) * (size_t)nx * py * pz);
#pragma omp parallel for schedule(static)
    for (int64_t jk = 0; jk < (int64_t)py * pz; ++jk)
        for (int32_t i = 0; i < nx; ++i) {
            double acc = 0.0;
            for (int32_t t = 0; t < W; ++t) acc += w[t] * a[jk * px + i + t];
            b[jk * nx + i] = acc;
        }
    /* along y: b (nx,py,pz) -> c (nx,ny,pz) */
    double *c = (double *)malloc(sizeof(double) * (size_t)nx * ny * pz);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < pz; ++k)
        for (int32_t j = 0; j < ny; ++j)
            for (int32_t i = 0; i < nx; ++i) {
                double acc = 0.0;
                for (int32_t t = 0; t < W; ++t) acc += w[t] * b[(k * py + j + t) * nx + i];
                c[(k * ny + j) * nx + i] = acc;
            }
    double norm = 1.0 / sqrt(w2 * w2 * w2);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nz; ++k)
        for (int32_t j = 0; j < ny; ++j)
            for (int32_t i = 0; i < nx; ++i) {
                double acc = 0.0;
                for (int32_t t = 0; t < W; ++t) acc += w[t] * c[((k + t) * ny + j) * nx + i];
                g[(k * ny + j) * nx + i] = acc * norm;
            }
    free(a); free(b); free(c); free(w);
}

/* Diffusion LDU from a cell field g: face conductivity k_f =
 * exp((g_owner + g_neighbour)/2), wall faces k = exp(g_cell) folded into the
 * diagonal (Dirichlet-0).  lower = upper = -k_f, diag = sum k.  k_bnd_sum
 * receives each cell's wall total so callers can rebuild diag from k. */
void wl_grid_diffusion_from_cells(int32_t nx, int32_t ny, int32_t nz,
                                   const double *g, double *k_face,
                                   double *k_bnd_sum, double *diag,
                                   double *lower, double *upper)
{
    int64_t n = (int64_t)nx * ny * nz, nf = wl_grid_n_faces(nx, ny, nz);
    int32_t *la = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nf > 0 ? nf : 1));
    int32_t *ua = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nf > 0 ? nf : 1));
    wl_grid_addressing(nx, ny, nz, la, ua);
    for (int64_t f = 0; f < nf; ++f) {
        k_face[f] = wl_exp(0.5 * (g[la[f]] + g[ua[f]]));
        lower[f] = -k_face[f];
        upper[f] = -k_face[f];
    }
    for (int64_t c = 0; c < n; ++c) {
        int32_t i = (int32_t)(c % nx), j = (int32_t)((c / nx) % ny), k = (int32_t)(c / ((int64_t)nx * ny));
        int nbf = n_boundary_faces(nx, ny, nz, i, j, k);
        k_bnd_sum[c] = (double)nbf * wl_exp(g[c]);
        diag[c] = k_bnd_sum[c];
    }
    for (int64_t f = 0; f < nf; ++f) { diag[la[f]] += k_face[f]; diag[ua[f]] += k_face[f]; }
    free(la); free(ua);
}

