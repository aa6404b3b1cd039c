/*
 * bso4_oracle.c -- CPU oracle (FP64) for the bispectrum-SO(4) descriptor-to-design-row path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of MILADY's algorithm,
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the checker.
 * The product (mld_gb300/, include/mld_gpu.h) never links, loads or calls it.
 *
 * Pinned against the reference's own golden vectors: tests/train_tests/fit17/REF/descDB/ (*.eml files)
 * (per-atom B, W bcc, j_max=4, r_cut=4.7) via tests/golden/fit17_bso4.npz.
 *
 * Reference files restated (paths inside the MILADY project):
 *   Clebsch-Gordan / Wigner-3j / factorial  src/mld/angular_functions.f90:432-546
 *   triple enumeration + flattened CG lists src/mld/compute/compute_bispectrum_so4.F90:740-918
 *   hyperspherical U^j and dU/dr recursion  src/mld/angular_functions.f90:41-273
 *   per-atom c^j, Z, B, dB                  src/mld/compute/compute_bispectrum_so4.F90:43-736,1014-1143
 *   sign convention of the derivative       src/mld/descriptors.F90:298-302
 *   cutoff functions                        src/mld/neighbours.F90:598-645
 *   neighbour lists (small / large box)     src/mld/neighbours.F90:186-364,787-847,1147-1328
 *   linear energy / force / stress rows     src/mld/mld_energy.F90:91-117,364-461,
 *                                           src/mld/mld_forces.F90:222-263,649-761,
 *                                           src/mld/mld_stress.F90:272-756
 *
 * Index conventions.  Angular momenta are doubled integers (j = 2*j_phys).  A layer j holds
 * (j+1)^2 complex entries U(p,q) with p,q in {-j,-j+2,...,j}; p is the first Fortran index
 * (Umm(m2,m1,j) -> p=m2, q=m1).  Flattened index: off[j] + ((p+j)/2)*(j+1) + (q+j)/2.
 * dB is returned with the post-flip sign of descriptors.F90:298-302, i.e. dB[n] = dB_k/du_n
 * where u_n = x_neighbour - x_centre.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

#define ORC_MAXJ 16

static int g_J = -1;              /* jj_max (doubled) */
static int g_K = 0;               /* number of (l1,l2,l) triples */
static int g_NU = 0;              /* sum_j (j+1)^2 */
static double g_inv_r0 = 0.0;     /* pi * inv_r0_input */
static int g_off[ORC_MAXJ + 2];
static int *g_tl1, *g_tl2, *g_tl;  /* triples in reference order */
static double *g_cgA, *g_cgB, *g_cgC;
static long g_nA, g_nB, g_nC;

static const double ONE_PI = 3.14159265358979323846264338327950288;

static inline int uidx(int j, int p, int q) { return g_off[j] + ((p + j) / 2) * (j + 1) + (q + j) / 2; }

/* angular_functions.f90:486-506 */
static double orc_factorial(int n) {
    double r = 1.0;
    for (int i = 2; i <= n; i++) r *= (double)i;
    return r;
}

static double ipow_m1(int e) { return (e % 2 == 0) ? 1.0 : -1.0; }

/* angular_functions.f90:451-483 (ntype = 2: all arguments doubled) */
static double orc_wigner3j(int j1, int m1, int j2, int m2, int j, int m) {
    const int nt = 2;
    double coef = ipow_m1((j1 - j2 - m) / nt) *
                  sqrt(orc_factorial((j1 + m1) / nt) * orc_factorial((j1 - m1) / nt) *
                       orc_factorial((j2 + m2) / nt) * orc_factorial((j2 - m2) / nt) *
                       orc_factorial((j + m) / nt) * orc_factorial((j - m) / nt));
    double tri = sqrt(orc_factorial((j1 + j2 - j) / nt) * orc_factorial((j1 - j2 + j) / nt) *
                      orc_factorial((-j1 + j2 + j) / nt) / orc_factorial((j1 + j2 + j) / nt + 1));
    int tmin = (j2 - j - m1) / nt;
    if ((j1 + m2 - j) / nt > tmin) tmin = (j1 + m2 - j) / nt;
    if (tmin < 0) tmin = 0;
    int tmax = (j1 + j2 - j) / nt;
    if ((j1 - m1) / nt < tmax) tmax = (j1 - m1) / nt;
    if ((j2 + m2) / nt < tmax) tmax = (j2 + m2) / nt;
    double s = 0.0;
    for (int t = tmin; t <= tmax; t++)
        s += ipow_m1(t) / (orc_factorial(t) * orc_factorial((j1 + j2 - j) / nt - t) *
                           orc_factorial((j1 - m1) / nt - t) * orc_factorial((j2 + m2) / nt - t) *
                           orc_factorial((j - j2 + m1) / nt + t) * orc_factorial((j - j1 - m2) / nt + t));
    return coef * tri * s;
}

/* angular_functions.f90:436-443 and the selection rules of compute_cg_vector :509-546 */
static double orc_cg(int j1, int m1, int j2, int m2, int j, int m) {
    if (m - m1 - m2 != 0) return 0.0;
    if (j1 + j2 - j < 0 || j - j1 + j2 < 0 || j - j2 + j1 < 0) return 0.0;
    if ((j + j1 + j2) % 2 == 1) return 0.0;
    if (m1 < -j1 || m1 > j1 || m2 < -j2 || m2 > j2 || m < -j || m > j) return 0.0;
    return ipow_m1((j1 - j2 + m) / 2) * sqrt(2.0 * (double)j / 2.0 + 1.0) * orc_wigner3j(j1, m1, j2, m2, j, -m);
}

static int imax(int a, int b) { return a > b ? a : b; }
static int imin(int a, int b) { return a < b ? a : b; }

/* compute_bispectrum_so4.F90:740-918: enumerate triples (l1, l2<=l1, l>=l1, parity even)
 * and flatten the CG products of the ZA/ZB/ZC contractions in loop order. */
int orc_init(double j_max, double inv_r0_input) {
    int J = (int)(2.0 * j_max);
    if (J < 0 || J > ORC_MAXJ) return -1;
    if (!(inv_r0_input > 0.0 && inv_r0_input < 1.0)) return -2;
    free(g_tl1); free(g_tl2); free(g_tl); free(g_cgA); free(g_cgB); free(g_cgC);
    g_J = J;
    g_inv_r0 = ONE_PI * inv_r0_input;
    g_NU = 0;
    for (int j = 0; j <= J; j++) { g_off[j] = g_NU; g_NU += (j + 1) * (j + 1); }
    g_off[J + 1] = g_NU;
    /* pass 1: count */
    int K = 0; long nA = 0, nB = 0, nC = 0;
    for (int l1 = 0; l1 <= J; l1++)
        for (int l2 = 0; l2 <= l1; l2++)
            for (int l = l1 - l2; l <= imin(J, l1 + l2); l++) {
                if ((l1 + l2 + l) % 2 == 1) continue;
                if (l < l1) continue;
                K++;
                for (int m1 = -l; m1 <= l; m1 += 2) for (int m2 = -l; m2 <= l; m2 += 2)
                    nA += (long)((imin(l1, m1 + l2) - imax(-l1, m1 - l2)) / 2 + 1) * ((imin(l1, m2 + l2) - imax(-l1, m2 - l2)) / 2 + 1);
                for (int m1 = -l1; m1 <= l1; m1 += 2) for (int m2 = -l1; m2 <= l1; m2 += 2)
                    nB += (long)((imin(l, m1 + l2) - imax(-l, m1 - l2)) / 2 + 1) * ((imin(l, m2 + l2) - imax(-l, m2 - l2)) / 2 + 1);
                for (int m1 = -l2; m1 <= l2; m1 += 2) for (int m2 = -l2; m2 <= l2; m2 += 2)
                    nC += (long)((imin(l1, m1 + l) - imax(-l1, m1 - l)) / 2 + 1) * ((imin(l1, m2 + l) - imax(-l1, m2 - l)) / 2 + 1);
            }
    g_K = K; g_nA = nA; g_nB = nB; g_nC = nC;
    g_tl1 = malloc(sizeof(int) * K); g_tl2 = malloc(sizeof(int) * K); g_tl = malloc(sizeof(int) * K);
    g_cgA = malloc(sizeof(double) * nA); g_cgB = malloc(sizeof(double) * nB); g_cgC = malloc(sizeof(double) * nC);
    int k = 0; long iA = 0, iB = 0, iC = 0;
    for (int l1 = 0; l1 <= J; l1++)
        for (int l2 = 0; l2 <= l1; l2++)
            for (int l = l1 - l2; l <= imin(J, l1 + l2); l++) {
                if ((l1 + l2 + l) % 2 == 1) continue;
                if (l < l1) continue;
                g_tl1[k] = l1; g_tl2[k] = l2; g_tl[k] = l; k++;
                for (int m1 = -l; m1 <= l; m1 += 2) for (int m2 = -l; m2 <= l; m2 += 2)
                    for (int ma = imax(-l1, m1 - l2); ma <= imin(l1, m1 + l2); ma += 2)
                        for (int mb = imax(-l1, m2 - l2); mb <= imin(l1, m2 + l2); mb += 2)
                            g_cgA[iA++] = orc_cg(l1, ma, l2, m1 - ma, l, m1) * orc_cg(l1, mb, l2, m2 - mb, l, m2);
                for (int m1 = -l1; m1 <= l1; m1 += 2) for (int m2 = -l1; m2 <= l1; m2 += 2)
                    for (int ma = imax(-l, m1 - l2); ma <= imin(l, m1 + l2); ma += 2)
                        for (int mb = imax(-l, m2 - l2); mb <= imin(l, m2 + l2); mb += 2)
                            g_cgB[iB++] = orc_cg(l, ma, l2, m1 - ma, l1, m1) * orc_cg(l, mb, l2, m2 - mb, l1, m2);
                for (int m1 = -l2; m1 <= l2; m1 += 2) for (int m2 = -l2; m2 <= l2; m2 += 2)
                    for (int ma = imax(-l1, m1 - l); ma <= imin(l1, m1 + l); ma += 2)
                        for (int mb = imax(-l1, m2 - l); mb <= imin(l1, m2 + l); mb += 2)
                            g_cgC[iC++] = orc_cg(l1, ma, l, m1 - ma, l2, m1) * orc_cg(l1, mb, l, m2 - mb, l2, m2);
            }
    return K;
}

int orc_num_triples(void) { return g_K; }
int orc_num_u(void) { return g_NU; }
long orc_num_cg(int which) { return which == 0 ? g_nA : which == 1 ? g_nB : g_nC; }
void orc_triples(int *l1, int *l2, int *l) {
    for (int k = 0; k < g_K; k++) { l1[k] = g_tl1[k]; l2[k] = g_tl2[k]; l[k] = g_tl[k]; }
}
/* 1-D Clebsch-Gordan coefficient (doubled indices), exported for table checks. */
double orc_cg_value(int j1, int m1, int j2, int m2, int j, int m) { return orc_cg(j1, m1, j2, m2, j, m); }

/* neighbours.F90:598-645 (types 2 and 3 used by the bispectrum path) */
static void orc_fcut(int type, double r, double rc, double width, double *f, double *df) {
    if (r > rc) { *f = 0.0; *df = 0.0; return; }
    if (type == 2) {
        double xx = r / rc;
        *f = 0.5 * (cos(ONE_PI * xx) + 1.0);
        *df = -0.5 * ONE_PI * sin(ONE_PI * xx) / rc;
    } else { /* type 3 */
        if (r < rc - width) { *f = 1.0; *df = 0.0; }
        else {
            double xx = ONE_PI * (r - rc + width) / width;
            *f = 0.5 * (cos(xx) + 1.0);
            *df = -0.5 * sin(xx) * ONE_PI / width;
        }
    }
}

/* angular_functions.f90:41-273 (spherical_4d).  Writes U (NU), and vec (3*NU) with
 * vec[a*NU + idx] = conj(U)*dfc*x_a/r + fc*conj(dU_a) -- the reference's class_mml%vecall. */
static void orc_spherical_4d(const double x[3], double rr, double rcut, double fc, double dfc,
                             cplx *U, cplx *dU /*3*NU scratch*/, cplx *vec, long vs) {
    const int NU = g_NU, J = g_J;
    double r0 = rcut / g_inv_r0;
    double th0 = rr / r0;
    double sin_i = 1.0 / sin(th0), tan_i = 1.0 / tan(th0);
    double l0 = rr * sin_i, l0i = 1.0 / l0, z0 = rr * tan_i;
    cplx zp = (z0 + I * x[2]) * l0i, zm = (z0 - I * x[2]) * l0i;
    cplx xp = (x[0] + I * x[1]) * l0i, xm = (x[0] - I * x[1]) * l0i;
    double drr[3] = {x[0] / rr, x[1] / rr, x[2] / rr};
    double dz = tan_i - th0 * sin_i * sin_i;
    double dil0 = (cos(th0) / r0 - l0i) / rr;
    cplx dzp[3], dzm[3], dxp[3], dxm[3];
    for (int a = 0; a < 3; a++) {
        dzp[a] = ((z0 + I * x[2]) * dil0 + dz * l0i) * drr[a];
        dzm[a] = ((z0 - I * x[2]) * dil0 + dz * l0i) * drr[a];
        dxp[a] = (x[0] + I * x[1]) * dil0 * drr[a];
        dxm[a] = (x[0] - I * x[1]) * dil0 * drr[a];
    }
    dzp[2] += I * l0i; dzm[2] -= I * l0i;
    dxp[0] += l0i; dxp[1] += I * l0i;
    dxm[0] += l0i; dxm[1] -= I * l0i;

    U[0] = 1.0;
    for (int a = 0; a < 3; a++) { dU[a * NU] = 0.0; vec[a] = dfc * drr[a]; }
    for (int j = 1; j <= J; j++) {
        for (int q = -j; q <= j; q += 2) {
            for (int p = -j; p <= j; p += 2) {
                cplx u = 0.0, du[3] = {0.0, 0.0, 0.0};
                if (q != -j) {
                    /* recursion from (q-1) column of layer j-1 */
                    double den = (double)(j + q);
                    if (p != -j) {  /* z_minus term uses (p-1, q-1) */
                        double t1 = sqrt((double)(j + p) / den);
                        int s = uidx(j - 1, p - 1, q - 1);
                        u += t1 * zm * U[s];
                        for (int a = 0; a < 3; a++) du[a] += t1 * (dzm[a] * U[s] + zm * dU[a * NU + s]);
                    }
                    if (p != j) {   /* x_plus term uses (p+1, q-1) */
                        cplx t2 = I * sqrt((double)(j - p) / den);
                        int s = uidx(j - 1, p + 1, q - 1);
                        u -= t2 * xp * U[s];
                        for (int a = 0; a < 3; a++) du[a] -= t2 * (dxp[a] * U[s] + xp * dU[a * NU + s]);
                    }
                } else {
                    /* q == -j: recursion from (q+1) column of layer j-1 */
                    double den = (double)(j - q);
                    if (p != j) {   /* z_plus term uses (p+1, q+1) */
                        double t2 = sqrt((double)(j - p) / den);
                        int s = uidx(j - 1, p + 1, q + 1);
                        u += t2 * zp * U[s];
                        for (int a = 0; a < 3; a++) du[a] += t2 * (dzp[a] * U[s] + zp * dU[a * NU + s]);
                    }
                    if (p != -j) {  /* x_minus term uses (p-1, q+1) */
                        cplx t1 = I * sqrt((double)(j + p) / den);
                        int s = uidx(j - 1, p - 1, q + 1);
                        u -= t1 * xm * U[s];
                        for (int a = 0; a < 3; a++) du[a] -= t1 * (dxm[a] * U[s] + xm * dU[a * NU + s]);
                    }
                }
                int d = uidx(j, p, q);
                U[d] = u;
                cplx cu = conj(u);
                for (int a = 0; a < 3; a++) {
                    dU[a * NU + d] = du[a];
                    vec[(long)d * vs + a] = cu * (dfc * drr[a]) + fc * conj(du[a]);
                }
            }
        }
    }
}

/* Reciprocal vectors b_k with a_i . b_k = delta_ik (ondm_recips). cell[3*i+c] = a_i[c]. */
static void orc_recips(const double *cell, double *bg) {
    const double *a1 = cell, *a2 = cell + 3, *a3 = cell + 6;
    double c23[3] = {a2[1] * a3[2] - a2[2] * a3[1], a2[2] * a3[0] - a2[0] * a3[2], a2[0] * a3[1] - a2[1] * a3[0]};
    double c31[3] = {a3[1] * a1[2] - a3[2] * a1[1], a3[2] * a1[0] - a3[0] * a1[2], a3[0] * a1[1] - a3[1] * a1[0]};
    double c12[3] = {a1[1] * a2[2] - a1[2] * a2[1], a1[2] * a2[0] - a1[0] * a2[2], a1[0] * a2[1] - a1[1] * a2[0]};
    double vol = a1[0] * c23[0] + a1[1] * c23[1] + a1[2] * c23[2];
    for (int c = 0; c < 3; c++) { bg[c] = c23[c] / vol; bg[3 + c] = c31[c] / vol; bg[6 + c] = c12[c] / vol; }
}

/* neighbours.F90:1331-1368 (|det|) */
double orc_volume(const double *cell) {
    const double *a1 = cell, *a2 = cell + 3, *a3 = cell + 6;
    double v = a1[0] * (a2[1] * a3[2] - a2[2] * a3[1]) - a1[1] * (a2[0] * a3[2] - a2[2] * a3[0]) +
               a1[2] * (a2[0] * a3[1] - a2[1] * a3[0]);
    return fabs(v);
}

/* neighbours.F90:787-847: small-box decision and image counts. */
int orc_small_box(const double *cell, double rcut, int nsize[3]) {
    double bg[9];
    orc_recips(cell, bg);
    int small = 0;
    for (int i = 0; i < 3; i++) {
        double bval = 1.0 / sqrt(bg[3 * i] * bg[3 * i] + bg[3 * i + 1] * bg[3 * i + 1] + bg[3 * i + 2] * bg[3 * i + 2]);
        int ncell = (int)(2.0 * rcut / bval) + 1;
        if (ncell > 1) small = 1;
        nsize[i] = ncell / 2 + 1;
    }
    return small;
}

/* Neighbour list of one structure within r < rcut.
 * small box: all periodic images within +-nsize (neighbours.F90:1147-1328 then the strict
 *            r < rcut filter of build_local_neighbours_ja :330);
 * large box: minimum image via nint of fractional components |ds|>0.5 (neighbours.F90:315-324).
 * u[(i*cap+n)*3+c] = x_neighbour - x_i.  Returns 0, or -1 if any atom exceeds cap. */
int orc_neighbours(int nat, const double *pos, const double *cell, double rcut, int cap,
                   int *nn, int *nbr, double *u, int *is_small) {
    int nsize[3];
    int small = orc_small_box(cell, rcut, nsize);
    *is_small = small;
    double bg[9];
    orc_recips(cell, bg);
    const double rc2 = rcut * rcut;
    int overflow = 0;
    for (int i = 0; i < nat; i++) {
        int c = 0;
        const double *xi = pos + 3 * i;
        if (small) {
            for (int jj = 0; jj < nat; jj++) {
                const double *xj = pos + 3 * jj;
                for (int n1 = -nsize[0]; n1 <= nsize[0]; n1++)
                    for (int n2 = -nsize[1]; n2 <= nsize[1]; n2++)
                        for (int n3 = -nsize[2]; n3 <= nsize[2]; n3++) {
                            double ut[3], r2 = 0.0;
                            for (int k = 0; k < 3; k++) {
                                ut[k] = xi[k] - (xj[k] + cell[k] * n1 + cell[3 + k] * n2 + cell[6 + k] * n3);
                                r2 += ut[k] * ut[k];
                            }
                            if (r2 < 1e-15) continue;
                            if (r2 > rc2) continue;
                            if (sqrt(r2) >= rcut) continue;
                            if (c < cap) {
                                nbr[i * cap + c] = jj;
                                for (int k = 0; k < 3; k++) u[(i * cap + c) * 3 + k] = -ut[k];
                            }
                            c++;
                        }
            }
        } else {
            for (int jj = 0; jj < nat; jj++) {
                if (jj == i) continue;
                const double *xj = pos + 3 * jj;
                double d[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
                double ds[3];
                for (int k = 0; k < 3; k++) {
                    ds[k] = d[0] * bg[3 * k] + d[1] * bg[3 * k + 1] + d[2] * bg[3 * k + 2];
                    if (ds[k] > 0.5 || ds[k] < -0.5) ds[k] -= round(ds[k]);
                }
                double dd[3], r2 = 0.0;
                for (int k = 0; k < 3; k++) {
                    dd[k] = cell[k] * ds[0] + cell[3 + k] * ds[1] + cell[6 + k] * ds[2];
                    r2 += dd[k] * dd[k];
                }
                if (sqrt(r2) >= rcut) continue;
                if (c < cap) {
                    nbr[i * cap + c] = jj;
                    for (int k = 0; k < 3; k++) u[(i * cap + c) * 3 + k] = dd[k];
                }
                c++;
            }
        }
        if (c > cap) { overflow = 1; c = cap; }
        nn[i] = c;
    }
    return overflow ? -1 : 0;
}

/* compute_bispectrum_so4.F90:43-736 + pack_cmm_into_ZcmmABC :1014-1143 for one structure.
 * chw[ch*ntypes + t]: neighbour weight of element t in channel ch (channel 0 = 1 for plain,
 *   channel 1 = weight_per_type, channel 2 = weight_per_type_3ch; compute_bispectrum_so4.F90:292-300,380-387).
 * rin[t1*ntypes+t2] > 0 switches on the inner cutoff (1 - f_in) of :356-377 (may be NULL).
 * B[(i*nch+ch)*K + k];  dB[((i*cap+n)*3+a)*nch*K + ch*K + k] (only if dB != NULL). */
int orc_bispectrum(int nat, const int *itype, int ntypes, int nch, const double *chw,
                   const double *rin, double rin_width, double rcut,
                   const int *nn, const int *nbr, const double *u, int cap,
                   double *B, double *dB) {
    (void)nbr;
    const int NU = g_NU, K = g_K, J = g_J;
    const int KK = nch * K;
    cplx *U = malloc(sizeof(cplx) * NU), *dUs = malloc(sizeof(cplx) * 3 * NU);
    const long vs = 3L * (cap > 0 ? cap : 1);   /* class_mml(m1,m2,j)%vecall(1:3n): vec[idx*vs + 3n + a] */
    cplx *vec = malloc(sizeof(cplx) * (size_t)vs * NU);
    cplx *dsum = malloc(sizeof(cplx) * (size_t)vs);
    double *nw = malloc(sizeof(double) * (size_t)nch * (cap > 0 ? cap : 1));
    cplx *cm = malloc(sizeof(cplx) * NU * nch);
    /* ZA/ZB/ZC stored per triple at offsets by layer sizes */
    long zsize = 0;
    for (int k = 0; k < K; k++) {
        int l1 = g_tl1[k], l2 = g_tl2[k], l = g_tl[k];
        zsize += (l + 1) * (l + 1) + (l1 + 1) * (l1 + 1) + (l2 + 1) * (l2 + 1);
    }
    cplx *Z = malloc(sizeof(cplx) * zsize * nch);
    for (int i = 0; i < nat; i++) {
        int n_i = nn[i];
        for (int ch = 0; ch < nch; ch++) for (int s = 0; s < NU; s++) cm[ch * NU + s] = 0.0;
        for (int n = 0; n < n_i; n++) {
            const double *x = u + (i * cap + n) * 3;
            double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            double fo, dfo, fi = 0.0, dfi = 0.0;
            orc_fcut(2, r, rcut, 0.0, &fo, &dfo);
            int tn = itype[nbr[i * cap + n]];
            if (rin) {
                double rci = rin[itype[i] * ntypes + tn];
                if (rci > 0.0) orc_fcut(3, r, rci + rin_width, rin_width, &fi, &dfi);
            }
            double fc = (1.0 - fi) * fo;
            double dfc = -dfi * fo + (1.0 - fi) * dfo;
            orc_spherical_4d(x, r, rcut, fc, dfc, U, dUs, vec + (size_t)n * 3, vs);
            for (int ch = 0; ch < nch; ch++) {
                double w = chw[ch * ntypes + tn];
                nw[ch * (cap > 0 ? cap : 1) + n] = w;
                double fw = fc * w;
                for (int s = 0; s < NU; s++) cm[ch * NU + s] += U[s] * fw;
            }
        }
        for (int ch = 0; ch < nch; ch++)
            for (int j = 0; j <= J; j++)
                for (int m = -j; m <= j; m += 2) cm[ch * NU + uidx(j, m, m)] += 1.0;
        /* Z contraction */
        for (int ch = 0; ch < nch; ch++) {
            const cplx *c = cm + ch * NU;
            cplx *z = Z + zsize * ch;
            long iA = 0, iB = 0, iC = 0, zo = 0;
            for (int k = 0; k < K; k++) {
                int l1 = g_tl1[k], l2 = g_tl2[k], l = g_tl[k];
                for (int m1 = -l; m1 <= l; m1 += 2) for (int m2 = -l; m2 <= l; m2 += 2) {
                    cplx s = 0.0;
                    for (int ma = imax(-l1, m1 - l2); ma <= imin(l1, m1 + l2); ma += 2)
                        for (int mb = imax(-l1, m2 - l2); mb <= imin(l1, m2 + l2); mb += 2)
                            s += g_cgA[iA++] * c[uidx(l1, ma, mb)] * c[uidx(l2, m1 - ma, m2 - mb)];
                    z[zo++] = s;
                }
                for (int m1 = -l1; m1 <= l1; m1 += 2) for (int m2 = -l1; m2 <= l1; m2 += 2) {
                    cplx s = 0.0;
                    for (int ma = imax(-l, m1 - l2); ma <= imin(l, m1 + l2); ma += 2)
                        for (int mb = imax(-l, m2 - l2); mb <= imin(l, m2 + l2); mb += 2)
                            s += g_cgB[iB++] * c[uidx(l, ma, mb)] * c[uidx(l2, m1 - ma, m2 - mb)];
                    z[zo++] = s;
                }
                for (int m1 = -l2; m1 <= l2; m1 += 2) for (int m2 = -l2; m2 <= l2; m2 += 2) {
                    cplx s = 0.0;
                    for (int ma = imax(-l1, m1 - l); ma <= imin(l1, m1 + l); ma += 2)
                        for (int mb = imax(-l1, m2 - l); mb <= imin(l1, m2 + l); mb += 2)
                            s += g_cgC[iC++] * c[uidx(l1, ma, mb)] * c[uidx(l, m1 - ma, m2 - mb)];
                    z[zo++] = s;
                }
            }
        }
        /* B and dB */
        for (int ch = 0; ch < nch; ch++) {
            const cplx *c = cm + ch * NU;
            const cplx *z = Z + zsize * ch;
            long zo = 0;
            for (int k = 0; k < K; k++) {
                int l1 = g_tl1[k], l2 = g_tl2[k], l = g_tl[k];
                const cplx *zA = z + zo, *zB = zA + (l + 1) * (l + 1), *zC = zB + (l1 + 1) * (l1 + 1);
                zo += (l + 1) * (l + 1) + (l1 + 1) * (l1 + 1) + (l2 + 1) * (l2 + 1);
                double e = 0.0;
                int t = 0;
                for (int m1 = -l; m1 <= l; m1 += 2) for (int m2 = -l; m2 <= l; m2 += 2, t++)
                    e += creal(conj(c[uidx(l, m1, m2)]) * zA[t]);
                B[((size_t)i * nch + ch) * K + k] = (n_i == 0) ? 0.0 : e;
                if (!dB) continue;
                double fB = (double)(1 + l) / (double)(1 + l1), fC = (double)(1 + l) / (double)(1 + l2);
                /* zaxpy over the contiguous 3n vecall of each (m1,m2,layer), as :560-690 */
                const int n3 = 3 * n_i;
                for (int e = 0; e < n3; e++) dsum[e] = 0.0;
                t = 0;
                for (int m1 = -l; m1 <= l; m1 += 2) for (int m2 = -l; m2 <= l; m2 += 2, t++) {
                    const cplx zz = zA[t];
                    const cplx *v = vec + (long)uidx(l, m1, m2) * vs;
                    for (int e = 0; e < n3; e++) dsum[e] += zz * v[e];
                }
                t = 0;
                for (int m1 = -l1; m1 <= l1; m1 += 2) for (int m2 = -l1; m2 <= l1; m2 += 2, t++) {
                    const cplx zz = zB[t] * fB;
                    const cplx *v = vec + (long)uidx(l1, m1, m2) * vs;
                    for (int e = 0; e < n3; e++) dsum[e] += zz * v[e];
                }
                t = 0;
                for (int m1 = -l2; m1 <= l2; m1 += 2) for (int m2 = -l2; m2 <= l2; m2 += 2, t++) {
                    const cplx zz = zC[t] * fC;
                    const cplx *v = vec + (long)uidx(l2, m1, m2) * vs;
                    for (int e = 0; e < n3; e++) dsum[e] += zz * v[e];
                }
                for (int n = 0; n < n_i; n++) {
                    /* vecall of a weighted channel is the plain one scaled by the neighbour weight */
                    double w = nw[ch * (cap > 0 ? cap : 1) + n];
                    for (int a = 0; a < 3; a++)
                        dB[(((size_t)i * cap + n) * 3 + a) * KK + (size_t)ch * K + k] = w * creal(dsum[3 * n + a]);
                }
            }
        }
    }
    free(U); free(dUs); free(vec); free(dsum); free(nw); free(cm); free(Z);
    return 0;
}

/* Linear design rows of one structure (D = 1 + KK):
 *   energy row  [nat, sum_i B_i]                                  (mld_energy.F90:91-117,364-461)
 *   3*nat force rows, atom-major x,y,z; col 0 = 0;
 *     row(ia) = -sum_i dB_i/dx_ia = sum_i [ sum_n dB_i(n) d(ia,i) - sum_n dB_i(n) d(ia,nbr_n) ]
 *                                                                  (mld_forces.F90:222-263,649-761)
 *   6 stress rows (xx,yy,zz,yz,xz,xy); col 0 = 0;
 *     sign_stress*3/V * sum_{i,n} dB_i(n)[alpha] * uu[beta] / r, with uu = x_n - x_i for a small
 *     box and uu = sign_stress_big_box*(x_i - x_n) for a large box  (mld_stress.F90:443-490,540-669,724-752)
 * rowE[D], rowF[3*nat*D], rowS[6*D]; any may be NULL. */
int orc_rows_linear(int nat, int KK, const double *B, const double *dB, const int *nn, const int *nbr,
                    const double *u, int cap, int is_small, double sign_stress, double sign_big, double volume,
                    double *rowE, double *rowF, double *rowS) {
    const int D = 1 + KK;
    static const int sa[6] = {0, 1, 2, 1, 0, 0}, sb[6] = {0, 1, 2, 2, 2, 1};
    if (rowE) {
        rowE[0] = (double)nat;
        for (int k = 0; k < KK; k++) {
            double s = 0.0;
            for (int i = 0; i < nat; i++) s += B[(size_t)i * KK + k];
            rowE[1 + k] = s;
        }
    }
    if (rowF) {
        memset(rowF, 0, sizeof(double) * (size_t)3 * nat * D);
        for (int i = 0; i < nat; i++)
            for (int n = 0; n < nn[i]; n++) {
                int ia = nbr[i * cap + n];
                for (int a = 0; a < 3; a++) {
                    const double *d = dB + (((size_t)i * cap + n) * 3 + a) * KK;
                    double *self = rowF + ((size_t)i * 3 + a) * D + 1;
                    double *other = rowF + ((size_t)ia * 3 + a) * D + 1;
                    for (int k = 0; k < KK; k++) { self[k] += d[k]; other[k] -= d[k]; }
                }
            }
    }
    if (rowS) {
        memset(rowS, 0, sizeof(double) * 6 * D);
        for (int i = 0; i < nat; i++)
            for (int n = 0; n < nn[i]; n++) {
                const double *x = u + ((size_t)i * cap + n) * 3;
                double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
                double uu[3];
                for (int c = 0; c < 3; c++) uu[c] = is_small ? x[c] : -sign_big * x[c];
                for (int s = 0; s < 6; s++) {
                    const double *d = dB + (((size_t)i * cap + n) * 3 + sa[s]) * KK;
                    double f = uu[sb[s]] / r;
                    for (int k = 0; k < KK; k++) rowS[s * D + 1 + k] += d[k] * f;
                }
            }
        double sc = sign_stress * 3.0 / volume;
        for (int s = 0; s < 6; s++) for (int k = 0; k < KK; k++) rowS[s * D + 1 + k] *= sc;
    }
    return 0;
}

/* Batch driver for the CPU baseline: neighbours + descriptors + linear design rows of many
 * structures, OpenMP-parallel over structures (the reference parallelises over configurations
 * with MPI subworlds, mld_mpi.F90:536-610).  Rows are written in the design-matrix order
 * E, 3*nat F, 6 S per structure: A[(row)*(1+KK) + col].  Returns 0 or the first error. */
int orc_rows_batch(int nstruct, const int *nat, const double *pos, const double *cell, const int *types,
                   int ntypes, int nch, const double *chw, double rcut, int cap,
                   double sign_stress, double sign_big, double *A) {
    const int K = g_K, KK = nch * K, D = 1 + KK;
    long *atom0 = malloc(sizeof(long) * (nstruct + 1));
    long *row0 = malloc(sizeof(long) * (nstruct + 1));
    atom0[0] = 0; row0[0] = 0;
    for (int s = 0; s < nstruct; s++) {
        atom0[s + 1] = atom0[s] + nat[s];
        row0[s + 1] = row0[s] + 1 + 3L * nat[s] + 6;
    }
    int err = 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int s = 0; s < nstruct; s++) {
        int n = nat[s];
        int *nn = malloc(sizeof(int) * n), *nb = malloc(sizeof(int) * (size_t)n * cap);
        double *u = malloc(sizeof(double) * (size_t)n * cap * 3);
        double *B = malloc(sizeof(double) * (size_t)n * KK);
        double *dB = malloc(sizeof(double) * (size_t)n * cap * 3 * KK);
        int small = 0;
        const double *cl = cell + 9L * s;
        if (orc_neighbours(n, pos + 3 * atom0[s], cl, rcut, cap, nn, nb, u, &small) != 0) {
#pragma omp atomic write
            err = 1;
        } else {
            orc_bispectrum(n, types + atom0[s], ntypes, nch, chw, NULL, 0.4, rcut, nn, nb, u, cap, B, dB);
            double *Ar = A + (size_t)row0[s] * D;
            orc_rows_linear(n, KK, B, dB, nn, nb, u, cap, small, sign_stress, sign_big, orc_volume(cl),
                            Ar, Ar + D, Ar + (size_t)(1 + 3 * n) * D);
        }
        free(nn); free(nb); free(u); free(B); free(dB);
    }
    free(atom0); free(row0);
    return err;
}

/* Quadratic (mld_order=2, QML full layout) design rows of one structure, D = 1 + KK + KK*KK:
 *   energy row   [nat, sum_i B_i, sum_i B_i (x) B_i]            (mld_energy.F90:170-266, :364-461;
 *                index of (id1,id2) = 1 + KK + KK*id1 + id2, 0-based)
 *   force rows   linear part as orc_rows_linear; quadratic part
 *                row(atom) -= sum_centres [f(id1) B_c(id2) + f(id2) B_c(id1)] with f the
 *                post-flip derivative force(:, c, n, :) and B_c the CENTRE's descriptor
 *                (mld_forces.F90:410-500)
 *   stress rows  sign_stress*3/V * sum_{i,n} [f(id1) B_nb(id2) + f(id2) B_nb(id1)] uu/r with B_nb
 *                the NEIGHBOUR's descriptor, as in mld_stress.F90:340-356/:580-603 where
 *                ik = kind_neigh(ia, ia_n). */
int orc_rows_quadratic(int nat, int KK, const double *B, const double *dB, const int *nn, const int *nbr,
                       const double *u, int cap, int is_small, double sign_stress, double sign_big, double volume,
                       double *rowE, double *rowF, double *rowS) {
    const int D = 1 + KK + KK * KK;
    static const int sa[6] = {0, 1, 2, 1, 0, 0}, sb[6] = {0, 1, 2, 2, 2, 1};
    if (rowE) {
        memset(rowE, 0, sizeof(double) * D);
        rowE[0] = (double)nat;
        for (int i = 0; i < nat; i++) {
            const double *b = B + (size_t)i * KK;
            for (int k = 0; k < KK; k++) rowE[1 + k] += b[k];
            for (int p = 0; p < KK; p++)
                for (int q = 0; q < KK; q++) rowE[1 + KK + KK * p + q] += b[p] * b[q];
        }
    }
    if (rowF) {
        memset(rowF, 0, sizeof(double) * (size_t)3 * nat * D);
        for (int i = 0; i < nat; i++) {
            const double *bc = B + (size_t)i * KK;
            for (int n = 0; n < nn[i]; n++) {
                int ia = nbr[i * cap + n];
                for (int a = 0; a < 3; a++) {
                    const double *d = dB + (((size_t)i * cap + n) * 3 + a) * KK;
                    double *self = rowF + ((size_t)i * 3 + a) * D;
                    double *other = rowF + ((size_t)ia * 3 + a) * D;
                    for (int k = 0; k < KK; k++) { self[1 + k] += d[k]; other[1 + k] -= d[k]; }
                    for (int p = 0; p < KK; p++)
                        for (int q = 0; q < KK; q++) {
                            double v = d[p] * bc[q] + d[q] * bc[p];
                            self[1 + KK + KK * p + q] += v;
                            other[1 + KK + KK * p + q] -= v;
                        }
                }
            }
        }
    }
    if (rowS) {
        memset(rowS, 0, sizeof(double) * 6 * D);
        for (int i = 0; i < nat; i++)
            for (int n = 0; n < nn[i]; n++) {
                const double *x = u + ((size_t)i * cap + n) * 3;
                const double *bn = B + (size_t)nbr[i * cap + n] * KK;
                double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
                double uu[3];
                for (int c = 0; c < 3; c++) uu[c] = is_small ? x[c] : -sign_big * x[c];
                for (int s = 0; s < 6; s++) {
                    const double *d = dB + (((size_t)i * cap + n) * 3 + sa[s]) * KK;
                    double f = uu[sb[s]] / r;
                    for (int k = 0; k < KK; k++) rowS[s * D + 1 + k] += d[k] * f;
                    for (int p = 0; p < KK; p++)
                        for (int q = 0; q < KK; q++) rowS[s * D + 1 + KK + KK * p + q] += (d[p] * bn[q] + d[q] * bn[p]) * f;
                }
            }
        double sc = sign_stress * 3.0 / volume;
        for (int s = 0; s < 6; s++) for (int k = 1; k < D; k++) rowS[s * D + k] *= sc;
    }
    return 0;
}

/* Kernel ridge design rows (ml_type = 1, polynomial kernel kernel_type = 4) of one structure,
 * D = 1 + KK + nk: columns [const, linear descriptor part, kernel part]
 * (mld_energy.F90:122-144, mld_forces.F90:268-320, mld_stress.F90:246-250,456,577).
 * Per atom x = B_i (raw) and reference point z_k (standardised, init_kernel in
 * compute_kernel.F90:1058-1256), inner_kernel_po (compute_kernel.F90:91-150):
 *   f(x,z) = (sigma2 + x.z/l2)^p, k = f / sqrt(f(x,x) f(z,z)), l2 = 2 length^2;
 *   per neighbour n and direction a, with g = force(:, i, n, a):
 *   dk = (p (sigma2 + x.z/l2)^(p-1)/l2 (g.z) - f * (g.x) * dker_xx / (2 f(x,x))) / sqrt(f(x,x) f(z,z)),
 *   dker_xx = 2 p (sigma2 + x.x/l2)^(p-1)/l2; force_kernel(k, i, 0) = -sum_n dk.
 * An atom without neighbours contributes zero kernel energy (compute_kernel.F90:747-749).
 * Packing follows the linear rows: row(i) += sum_n dk, row(nbr) -= dk; stress rows from the
 * per-pair dk with uu/r as in orc_rows_linear. */
int orc_rows_kernel(int nat, int KK, const double *B, const double *dB, const int *nn, const int *nbr,
                    const double *u, int cap, int is_small, double sign_stress, double sign_big, double volume,
                    int nk, const double *Z, double power, double length, double sigma,
                    double *rowE, double *rowF, double *rowS) {
    const int D = 1 + KK + nk, c0 = 1 + KK;
    static const int sa[6] = {0, 1, 2, 1, 0, 0}, sb[6] = {0, 1, 2, 2, 2, 1};
    const double l2 = 2.0 * length * length, s2 = sigma * sigma;
    /* linear part first (also zeroes the rows) */
    double *tE = rowE ? malloc(sizeof(double) * (1 + KK)) : NULL;
    double *tF = rowF ? malloc(sizeof(double) * (size_t)3 * nat * (1 + KK)) : NULL;
    double *tS = rowS ? malloc(sizeof(double) * 6 * (1 + KK)) : NULL;
    orc_rows_linear(nat, KK, B, dB, nn, nbr, u, cap, is_small, sign_stress, sign_big, volume, tE, tF, tS);
    if (rowE) { memset(rowE, 0, sizeof(double) * D); memcpy(rowE, tE, sizeof(double) * (1 + KK)); }
    if (rowF) {
        memset(rowF, 0, sizeof(double) * (size_t)3 * nat * D);
        for (long r = 0; r < 3L * nat; r++) memcpy(rowF + r * D, tF + r * (1 + KK), sizeof(double) * (1 + KK));
    }
    if (rowS) {
        memset(rowS, 0, sizeof(double) * 6 * D);
        for (int r = 0; r < 6; r++) memcpy(rowS + r * D, tS + r * (1 + KK), sizeof(double) * (1 + KK));
    }
    free(tE); free(tF); free(tS);
    double *zz = malloc(sizeof(double) * nk);
    for (int k = 0; k < nk; k++) {
        double s = 0.0;
        for (int c = 0; c < KK; c++) s += Z[(size_t)k * KK + c] * Z[(size_t)k * KK + c];
        zz[k] = pow(s2 + s / l2, power);  /* f(z,z) */
    }
    double *gx = malloc(sizeof(double) * 3), *Sk = calloc((size_t)6 * nk, sizeof(double));
    for (int i = 0; i < nat; i++) {
        if (nn[i] == 0) continue;
        const double *x = B + (size_t)i * KK;
        double xx = 0.0;
        for (int c = 0; c < KK; c++) xx += x[c] * x[c];
        const double kxx = pow(s2 + xx / l2, power), skxx = sqrt(kxx);
        const double dkxx = 2.0 * power * pow(s2 + xx / l2, power - 1.0) / l2;
        for (int k = 0; k < nk; k++) {
            const double *z = Z + (size_t)k * KK;
            double xz = 0.0;
            for (int c = 0; c < KK; c++) xz += x[c] * z[c];
            const double base = s2 + xz / l2;
            const double kt = pow(base, power);
            const double aaa = sqrt(zz[k]) * skxx, bbb = 2.0 * kxx;
            if (rowE) rowE[c0 + k] += kt / aaa;
            const double tf1 = power * pow(base, power - 1.0) / l2;
            for (int n = 0; n < nn[i]; n++) {
                const int ia = nbr[i * cap + n];
                const double *xn = u + ((size_t)i * cap + n) * 3;
                const double r = sqrt(xn[0] * xn[0] + xn[1] * xn[1] + xn[2] * xn[2]);
                double dk[3];
                for (int a = 0; a < 3; a++) {
                    const double *g = dB + (((size_t)i * cap + n) * 3 + a) * KK;
                    double gz = 0.0, gxv = 0.0;
                    for (int c = 0; c < KK; c++) { gz += g[c] * z[c]; gxv += g[c] * x[c]; }
                    dk[a] = (tf1 * gz - kt * gxv * dkxx / bbb) / aaa;
                    if (rowF) {
                        rowF[((size_t)i * 3 + a) * D + c0 + k] += dk[a];
                        rowF[((size_t)ia * 3 + a) * D + c0 + k] -= dk[a];
                    }
                }
                if (rowS) {
                    double uu[3];
                    for (int c = 0; c < 3; c++) uu[c] = is_small ? xn[c] : -sign_big * xn[c];
                    for (int s = 0; s < 6; s++) Sk[(size_t)s * nk + k] += dk[sa[s]] * uu[sb[s]] / r;
                }
            }
        }
    }
    if (rowS) {
        const double sc = sign_stress * 3.0 / volume;
        for (int s = 0; s < 6; s++) for (int k = 0; k < nk; k++) rowS[s * D + c0 + k] = sc * Sk[(size_t)s * nk + k];
    }
    free(zz); free(gx); free(Sk);
    return 0;
}
