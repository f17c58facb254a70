/*
 * pq2_port.c -- CPU ORACLE (test infrastructure only; never shipped, never on
 * the product path).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs load the shared object built from this file.
 *
 * A restatement, in plain C, of the reference's integral library and of its
 * matrix builders:
 *   - THO-1966 primitive ERI          libpyquante2/cints.c:72-149
 *   - NR incomplete-gamma Boys        libpyquante2/cints.c:302-373
 *   - THO overlap / kinetic / nuclear libpyquante2/cints.c:152-269
 *   - helpers                         libpyquante2/cints.c:272-300,375-395
 *   - S/T/V, JK_direct, build_I,
 *     JK_inmem matrix semantics       src/basis.rs:214-484
 *   - J/K with 8-fold symmetry and a Schwarz screen over contracted
 *     functions (the strong CPU baseline of the Fock build; same integrals)
 *   - multipole moments               src/integrals/os86.rs:775-828 (restated
 *                                     through 1-D overlaps, not the symbolic
 *                                     expansion)
 *
 * Parity of this port is pinned two ways: against the os86/tho66 golden
 * vectors (tests/golden) and, where the reference C sources are present, against
 * the reference library itself compiled by oracle/Makefile (make -C oracle ref).
 *
 * Boys function modes (oq_set_boys_mode):
 *   0 = "as shipped": the Numerical-Recipes series / continued fraction with
 *       EPS 3e-7 and the x >= 1e-8 clamp (relative error ~1e-7);
 *   1 = exact: power series for x < 35, erf + upward recursion above
 *       (relative error ~1e-16).  This is the 1e-12-per-integral oracle.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* integer helpers (cints.c:272-300,389)                                     */
/* ------------------------------------------------------------------------ */
static double ofact(int n) { double r = 1.0; for (int i = 2; i <= n; ++i) r *= i; return r; }
static double ofact2(int n) { double r = 1.0; for (int i = n; i > 1; i -= 2) r *= i; return r; }
static double obinom(int a, int b) {
    if (b < 0 || b > a) return 0.0;
    return ofact(a) / (ofact(b) * ofact(a - b));
}
/* a! / (b! (a-2b)!)  -- cints.c:389 */
static double ofact_ratio2(int a, int b) { return ofact(a) / ofact(b) / ofact(a - 2 * b); }
static double oipow(double x, int n) {
    double r = 1.0;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

/* Coefficient of x^s in (x+xpa)^ia (x+xpb)^ib  -- cints.c:291-298 */
static double obinomial_prefactor(int s, int ia, int ib, double xpa, double xpb) {
    double sum = 0.0;
    for (int t = 0; t <= s; ++t) {
        if (s - ia <= t && t <= ib)
            sum += obinom(ia, s - t) * obinom(ib, t) * oipow(xpa, ia - s + t) * oipow(xpb, ib - t);
    }
    return sum;
}

/* ------------------------------------------------------------------------ */
/* Boys function                                                             */
/* ------------------------------------------------------------------------ */
static int g_boys_exact = 1;
void oq_set_boys_mode(int exact) { g_boys_exact = exact ? 1 : 0; }
int oq_get_boys_mode(void) { return g_boys_exact; }

/* Lower incomplete gamma gamma(a, x) by the Numerical-Recipes series (x < a+1)
 * or modified-Lentz continued fraction; EPS 3e-7, 100 iterations.
 * cints.c:310-373 (gamm_inc / gser / gcf). */
static double nr_lower_gamma(double a, double x) {
    const double eps = 3.0e-7, fpmin = 1.0e-30;
    const int itmax = 100;
    double gln = lgamma(a);
    if (x < a + 1.0) {
        if (x <= 0.0) return 0.0;
        double ap = a, del = 1.0 / a, sum = del;
        for (int n = 1; n <= itmax; ++n) {
            ap += 1.0;
            del *= x / ap;
            sum += del;
            if (fabs(del) < fabs(sum) * eps) break;
        }
        return exp(gln) * (sum * exp(-x + a * log(x) - gln));
    }
    double b = x + 1.0 - a, c = 1.0 / fpmin, d = 1.0 / b, h = d;
    for (int i = 1; i <= itmax; ++i) {
        double an = -i * (i - a);
        b += 2.0;
        d = an * d + b;
        if (fabs(d) < fpmin) d = fpmin;
        c = b + an / c;
        if (fabs(c) < fpmin) c = fpmin;
        d = 1.0 / d;
        double del = d * c;
        h *= del;
        if (fabs(del - 1.0) < eps) break;
    }
    return exp(gln) * (1.0 - exp(-x + a * log(x) - gln) * h);
}

/* F_m(x) as the reference ships it: x clamped to >= 1e-8 -- cints.c:302-308 */
double oq_fgamma_nr(double m, double x) {
    if (fabs(x) < 1.0e-8) x = 1.0e-8;
    return 0.5 * pow(x, -m - 0.5) * nr_lower_gamma(m + 0.5, x);
}

/* Exact F_m(x) = int_0^1 t^{2m} exp(-x t^2) dt.
 * x < 35: F_m = e^{-x} sum_k (2x)^k / prod_{i=0..k}(2m+2i+1)  (all terms > 0);
 * x >= 35: F_0 = sqrt(pi/x) erf(sqrt x) / 2, F_{k+1} = ((2k+1)F_k - e^{-x})/(2x),
 * which is stable upward because x > m. */
double oq_boys_exact(int m, double x) {
    if (x < 0.0) x = 0.0;
    if (x < 35.0) {
        double term = 1.0 / (2 * m + 1), sum = term;
        for (int k = 1; k < 500; ++k) {
            term *= 2.0 * x / (2 * m + 2 * k + 1);
            sum += term;
            if (term < sum * 1.0e-18) break;
        }
        return exp(-x) * sum;
    }
    double e = exp(-x);
    double f = 0.5 * sqrt(M_PI / x) * erf(sqrt(x));
    for (int k = 0; k < m; ++k) f = ((2 * k + 1) * f - e) / (2.0 * x);
    return f;
}

/* cints-signature Boys entry: dispatches on the mode. */
double oq_fgamma(double m, double x) {
    if (g_boys_exact) return oq_boys_exact((int)(m + 0.5), x);
    return oq_fgamma_nr(m, x);
}

/* ------------------------------------------------------------------------ */
/* THO primitive ERI -- cints.c:72-149 (eq. 2.22)                            */
/* ------------------------------------------------------------------------ */
/* One Cartesian direction of the THO expansion: B[I], I = 0..l1+l2+l3+l4.
 * Same sums as cints.c:117-149 (B_array / B_term / fB / Bfunc), kept on the
 * stack instead of malloc'd. */
static void tho_B(int l1, int l2, int l3, int l4, double p, double a, double b,
                  double q, double c, double d, double g1, double g2, double delta,
                  double *B) {
    int imax = l1 + l2 + l3 + l4 + 1;
    for (int i = 0; i < imax; ++i) B[i] = 0.0;
    for (int i1 = 0; i1 <= l1 + l2; ++i1) {
        double bp1 = obinomial_prefactor(i1, l1, l2, p - a, p - b);
        for (int i2 = 0; i2 <= l3 + l4; ++i2) {
            double bp2 = obinomial_prefactor(i2, l3, l4, q - c, q - d);
            double sgn2 = (i2 & 1) ? -1.0 : 1.0;
            for (int r1 = 0; r1 <= i1 / 2; ++r1) {
                double f1 = bp1 * ofact_ratio2(i1, r1) / oipow(4.0 * g1, i1 - r1);
                for (int r2 = 0; r2 <= i2 / 2; ++r2) {
                    double f2 = sgn2 * bp2 * ofact_ratio2(i2, r2) / oipow(4.0 * g2, i2 - r2);
                    int s = i1 + i2 - 2 * (r1 + r2);
                    for (int u = 0; u <= s / 2; ++u) {
                        double sgnu = (u & 1) ? -1.0 : 1.0;
                        double t = f1 * f2 * sgnu * ofact_ratio2(s, u) *
                                   oipow(q - p, s - 2 * u) / oipow(delta, s - u);
                        B[s - u] += t;
                    }
                }
            }
        }
    }
}

double oq_coulomb_repulsion(double xa, double ya, double za, double norma, int la, int ma, int na, double alphaa,
                            double xb, double yb, double zb, double normb, int lb, int mb, int nb, double alphab,
                            double xc, double yc, double zc, double normc, int lc, int mc, int nc, double alphac,
                            double xd, double yd, double zd, double normd, int ld, int md, int nd, double alphad) {
    double rab2 = (xa - xb) * (xa - xb) + (ya - yb) * (ya - yb) + (za - zb) * (za - zb);
    double rcd2 = (xc - xd) * (xc - xd) + (yc - yd) * (yc - yd) + (zc - zd) * (zc - zd);
    double g1 = alphaa + alphab, g2 = alphac + alphad;
    double xp = (alphaa * xa + alphab * xb) / g1, yp = (alphaa * ya + alphab * yb) / g1,
           zp = (alphaa * za + alphab * zb) / g1;
    double xq = (alphac * xc + alphad * xd) / g2, yq = (alphac * yc + alphad * yd) / g2,
           zq = (alphac * zc + alphad * zd) / g2;
    double rpq2 = (xp - xq) * (xp - xq) + (yp - yq) * (yp - yq) + (zp - zq) * (zp - zq);
    double delta = (1.0 / g1 + 1.0 / g2) / 4.0;
    double Bx[32], By[32], Bz[32];
    tho_B(la, lb, lc, ld, xp, xa, xb, xq, xc, xd, g1, g2, delta, Bx);
    tho_B(ma, mb, mc, md, yp, ya, yb, yq, yc, yd, g1, g2, delta, By);
    tho_B(na, nb, nc, nd, zp, za, zb, zq, zc, zd, g1, g2, delta, Bz);
    double T = 0.25 * rpq2 / delta;
    double sum = 0.0;
    /* one Boys call per (I,J,K) term, as the reference does (cints.c:103-106) */
    for (int I = 0; I <= la + lb + lc + ld; ++I)
        for (int J = 0; J <= ma + mb + mc + md; ++J)
            for (int K = 0; K <= na + nb + nc + nd; ++K)
                sum += Bx[I] * By[J] * Bz[K] * oq_fgamma((double)(I + J + K), T);
    return 2.0 * pow(M_PI, 2.5) / (g1 * g2 * sqrt(g1 + g2)) * exp(-alphaa * alphab * rab2 / g1) *
           exp(-alphac * alphad * rcd2 / g2) * sum * norma * normb * normc * normd;
}

/* ------------------------------------------------------------------------ */
/* one-electron integrals -- cints.c:152-269                                 */
/* ------------------------------------------------------------------------ */
/* THO eq. 2.12, cints.c:198-208 */
static double tho_overlap_1d(int l1, int l2, double pax, double pbx, double g) {
    if (l1 < 0 || l2 < 0) return 0.0;
    double sum = 0.0;
    for (int i = 0; i <= (l1 + l2) / 2; ++i)
        sum += obinomial_prefactor(2 * i, l1, l2, pax, pbx) * ofact2(2 * i - 1) / oipow(2.0 * g, i);
    return sum;
}

/* cints.c:177-196 (unnormalised) */
double oq_overlap(double alpha1, int l1, int m1, int n1, double xa, double ya, double za,
                  double alpha2, int l2, int m2, int n2, double xb, double yb, double zb) {
    double g = alpha1 + alpha2;
    double rab2 = (xa - xb) * (xa - xb) + (ya - yb) * (ya - yb) + (za - zb) * (za - zb);
    double xp = (alpha1 * xa + alpha2 * xb) / g, yp = (alpha1 * ya + alpha2 * yb) / g,
           zp = (alpha1 * za + alpha2 * zb) / g;
    double pre = pow(M_PI / g, 1.5) * exp(-alpha1 * alpha2 * rab2 / g);
    return pre * tho_overlap_1d(l1, l2, xp - xa, xp - xb, g) * tho_overlap_1d(m1, m2, yp - ya, yp - yb, g) *
           tho_overlap_1d(n1, n2, zp - za, zp - zb, g);
}

/* cints.c:152-175: T via overlaps with the ket powers raised / lowered by 2 */
double oq_kinetic(double alpha1, int l1, int m1, int n1, double xa, double ya, double za,
                  double alpha2, int l2, int m2, int n2, double xb, double yb, double zb) {
#define OVL(L2, M2, N2) oq_overlap(alpha1, l1, m1, n1, xa, ya, za, alpha2, (L2), (M2), (N2), xb, yb, zb)
    double t0 = alpha2 * (2 * (l2 + m2 + n2) + 3) * OVL(l2, m2, n2);
    double t1 = -2.0 * alpha2 * alpha2 * (OVL(l2 + 2, m2, n2) + OVL(l2, m2 + 2, n2) + OVL(l2, m2, n2 + 2));
    double t2 = 0.0;
    if (l2 > 1) t2 += l2 * (l2 - 1) * OVL(l2 - 2, m2, n2);
    if (m2 > 1) t2 += m2 * (m2 - 1) * OVL(l2, m2 - 2, n2);
    if (n2 > 1) t2 += n2 * (n2 - 1) * OVL(l2, m2, n2 - 2);
#undef OVL
    return t0 + t1 - 0.5 * t2;
}

/* THO eq. 2.18 / 3.1, cints.c:245-269 */
static void tho_A(int l1, int l2, double pa, double pb, double cp, double g, double *A) {
    int imax = l1 + l2 + 1;
    for (int i = 0; i < imax; ++i) A[i] = 0.0;
    for (int i = 0; i < imax; ++i) {
        double bp = obinomial_prefactor(i, l1, l2, pa, pb);
        double sgni = (i & 1) ? -1.0 : 1.0;
        for (int r = 0; r <= i / 2; ++r)
            for (int u = 0; u <= (i - 2 * r) / 2; ++u) {
                double sgnu = (u & 1) ? -1.0 : 1.0;
                int k = i - 2 * r - 2 * u;
                A[i - 2 * r - u] += sgni * bp * sgnu * ofact(i) * oipow(cp, k) * oipow(0.25 / g, r + u) /
                                    (ofact(r) * ofact(u) * ofact(k));
            }
    }
}

/* cints.c:210-243 (includes the norms and the minus sign) */
double oq_nuclear_attraction(double x1, double y1, double z1, double norm1, int l1, int m1, int n1, double alpha1,
                             double x2, double y2, double z2, double norm2, int l2, int m2, int n2, double alpha2,
                             double x3, double y3, double z3) {
    double g = alpha1 + alpha2;
    double xp = (alpha1 * x1 + alpha2 * x2) / g, yp = (alpha1 * y1 + alpha2 * y2) / g,
           zp = (alpha1 * z1 + alpha2 * z2) / g;
    double rab2 = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2) + (z1 - z2) * (z1 - z2);
    double rcp2 = (x3 - xp) * (x3 - xp) + (y3 - yp) * (y3 - yp) + (z3 - zp) * (z3 - zp);
    double Ax[16], Ay[16], Az[16];
    tho_A(l1, l2, xp - x1, xp - x2, xp - x3, g, Ax);
    tho_A(m1, m2, yp - y1, yp - y2, yp - y3, g, Ay);
    tho_A(n1, n2, zp - z1, zp - z2, zp - z3, g, Az);
    double sum = 0.0;
    for (int I = 0; I <= l1 + l2; ++I)
        for (int J = 0; J <= m1 + m2; ++J)
            for (int K = 0; K <= n1 + n2; ++K)
                sum += Ax[I] * Ay[J] * Az[K] * oq_fgamma((double)(I + J + K), rcp2 * g);
    return -norm1 * norm2 * 2.0 * M_PI / g * exp(-alpha1 * alpha2 * rab2 / g) * sum;
}

/* Multipole moment <a| (x-Cx)^ox (y-Cy)^oy (z-Cz)^oz |b>, unnormalised, the
 * quantity of os86.rs:775-828.  (x-Cx)^k = sum_j C(k,j) (Bx-Cx)^(k-j) (x-Bx)^j,
 * so each direction is a short sum of 1-D overlaps with the b power raised. */
double oq_moment(double alpha1, int l1, int m1, int n1, double xa, double ya, double za,
                 double alpha2, int l2, int m2, int n2, double xb, double yb, double zb,
                 double xc, double yc, double zc, int ox, int oy, int oz) {
    double g = alpha1 + alpha2;
    double rab2 = (xa - xb) * (xa - xb) + (ya - yb) * (ya - yb) + (za - zb) * (za - zb);
    double P[3] = {(alpha1 * xa + alpha2 * xb) / g, (alpha1 * ya + alpha2 * yb) / g, (alpha1 * za + alpha2 * zb) / g};
    double A[3] = {xa, ya, za}, B[3] = {xb, yb, zb}, C[3] = {xc, yc, zc};
    int la[3] = {l1, m1, n1}, lb[3] = {l2, m2, n2}, o[3] = {ox, oy, oz};
    double pre = pow(M_PI / g, 1.5) * exp(-alpha1 * alpha2 * rab2 / g);
    for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int j = 0; j <= o[d]; ++j)
            s += obinom(o[d], j) * oipow(B[d] - C[d], o[d] - j) *
                 tho_overlap_1d(la[d], lb[d] + j, P[d] - A[d], P[d] - B[d], g);
        pre *= s;
    }
    return pre;
}

/* ------------------------------------------------------------------------ */
/* matrix builders -- src/basis.rs:116-484                                   */
/* ------------------------------------------------------------------------ */
/* A basis is n contracted Cartesian functions (CGTOs, basis.rs:152-173):
 *   origin[3n], powers[3n], nprim[n], prim_off[n] into exps/coefs/norms.
 * norms[] holds the per-primitive normalisation of basis.rs:140-149. */
typedef double (*oq_eri_fn)(double, double, double, double, int, int, int, double,
                            double, double, double, double, int, int, int, double,
                            double, double, double, double, int, int, int, double,
                            double, double, double, double, int, int, int, double);
typedef double (*oq_ovl_fn)(double, int, int, int, double, double, double,
                            double, int, int, int, double, double, double);
typedef double (*oq_nuc_fn)(double, double, double, double, int, int, int, double,
                            double, double, double, double, int, int, int, double,
                            double, double, double);

typedef struct {
    int n;
    const double *origin;
    const int *powers;
    const int *nprim;
    const int *prim_off;
    const double *exps, *coefs, *norms;
} oq_basis;

/* PGTO::normalization, basis.rs:140-149 */
double oq_pgto_norm(double alpha, int l, int m, int n) {
    int L = l + m + n;
    double num = pow(2.0, 2.0 * L + 1.5) * pow(alpha, L + 1.5);
    double den = ofact2(2 * l - 1) * ofact2(2 * m - 1) * ofact2(2 * n - 1) * pow(M_PI, 1.5);
    return sqrt(num / den);
}

static double prim_eri(oq_eri_fn f, const oq_basis *b, int i, int pi, int j, int pj, int k, int pk, int l, int pl) {
    const double *A = b->origin + 3 * i, *B = b->origin + 3 * j, *C = b->origin + 3 * k, *D = b->origin + 3 * l;
    const int *a = b->powers + 3 * i, *bb = b->powers + 3 * j, *c = b->powers + 3 * k, *d = b->powers + 3 * l;
    return f(A[0], A[1], A[2], b->norms[pi], a[0], a[1], a[2], b->exps[pi],
             B[0], B[1], B[2], b->norms[pj], bb[0], bb[1], bb[2], b->exps[pj],
             C[0], C[1], C[2], b->norms[pk], c[0], c[1], c[2], b->exps[pk],
             D[0], D[1], D[2], b->norms[pl], d[0], d[1], d[2], b->exps[pl]);
}

/* contracted (ij|kl): sum over K^4 primitives of c c c c (ab|cd) -- basis.rs:441-450 */
static double contr_eri(oq_eri_fn f, const oq_basis *b, int i, int j, int k, int l) {
    double v = 0.0;
    for (int a = 0; a < b->nprim[i]; ++a) {
        int pa = b->prim_off[i] + a;
        for (int bb = 0; bb < b->nprim[j]; ++bb) {
            int pb = b->prim_off[j] + bb;
            for (int c = 0; c < b->nprim[k]; ++c) {
                int pc = b->prim_off[k] + c;
                for (int d = 0; d < b->nprim[l]; ++d) {
                    int pd = b->prim_off[l] + d;
                    v += b->coefs[pa] * b->coefs[pb] * b->coefs[pc] * b->coefs[pd] *
                         prim_eri(f, b, i, pa, j, pb, k, pc, l, pd);
                }
            }
        }
    }
    return v;
}

#define OQ_BASIS_ARGS int n, const double *origin, const int *powers, const int *nprim, const int *prim_off, \
                      const double *exps, const double *coefs, const double *norms
#define OQ_BASIS_INIT oq_basis bs = {n, origin, powers, nprim, prim_off, exps, coefs, norms}

double oq_contracted_eri(OQ_BASIS_ARGS, void *eri, int i, int j, int k, int l) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
    return contr_eri(f, &bs, i, j, k, l);
}

/* S and T: lower triangle + mirror, basis.rs:214-290 */
static void one_e(const oq_basis *b, oq_ovl_fn f, double *out) {
    for (int mu = 0; mu < b->n; ++mu)
        for (int nu = 0; nu <= mu; ++nu) {
            const double *A = b->origin + 3 * mu, *B = b->origin + 3 * nu;
            const int *a = b->powers + 3 * mu, *c = b->powers + 3 * nu;
            double v = 0.0;
            for (int q = 0; q < b->nprim[nu]; ++q) {
                int pb = b->prim_off[nu] + q;
                double inner = 0.0;
                for (int p = 0; p < b->nprim[mu]; ++p) {
                    int pa = b->prim_off[mu] + p;
                    inner += b->coefs[pa] * b->norms[pa] * b->norms[pb] *
                             f(b->exps[pa], a[0], a[1], a[2], A[0], A[1], A[2],
                               b->exps[pb], c[0], c[1], c[2], B[0], B[1], B[2]);
                }
                v += b->coefs[pb] * inner;
            }
            out[mu * b->n + nu] = v;
            out[nu * b->n + mu] = v;
        }
}

void oq_S(OQ_BASIS_ARGS, void *ovl, double *out) {
    OQ_BASIS_INIT;
    one_e(&bs, ovl ? (oq_ovl_fn)ovl : oq_overlap, out);
}
void oq_T(OQ_BASIS_ARGS, void *kin, double *out) {
    OQ_BASIS_INIT;
    one_e(&bs, kin ? (oq_ovl_fn)kin : oq_kinetic, out);
}

/* V = sum_C Z_C V_C, basis.rs:316-338 */
void oq_V(OQ_BASIS_ARGS, void *nuc, int natoms, const double *Z, const double *coords, double *out) {
    OQ_BASIS_INIT;
    oq_nuc_fn f = nuc ? (oq_nuc_fn)nuc : oq_nuclear_attraction;
    for (int i = 0; i < n * n; ++i) out[i] = 0.0;
    for (int c = 0; c < natoms; ++c) {
        const double *R = coords + 3 * c;
        for (int mu = 0; mu < n; ++mu)
            for (int nu = 0; nu <= mu; ++nu) {
                const double *A = bs.origin + 3 * mu, *B = bs.origin + 3 * nu;
                const int *a = bs.powers + 3 * mu, *bb = bs.powers + 3 * nu;
                double v = 0.0;
                for (int q = 0; q < bs.nprim[nu]; ++q) {
                    int pb = bs.prim_off[nu] + q;
                    double inner = 0.0;
                    for (int p = 0; p < bs.nprim[mu]; ++p) {
                        int pa = bs.prim_off[mu] + p;
                        inner += bs.coefs[pa] * f(A[0], A[1], A[2], bs.norms[pa], a[0], a[1], a[2], bs.exps[pa],
                                                  B[0], B[1], B[2], bs.norms[pb], bb[0], bb[1], bb[2], bs.exps[pb],
                                                  R[0], R[1], R[2]);
                    }
                    v += bs.coefs[pb] * inner;
                }
                out[mu * n + nu] += Z[c] * v;
                if (nu != mu) out[nu * n + mu] += Z[c] * v;
            }
    }
}

/* Multipole-moment matrix about C with orders (ox,oy,oz), normalised like S. */
void oq_M(OQ_BASIS_ARGS, const double *C, int ox, int oy, int oz, double *out) {
    OQ_BASIS_INIT;
    for (int mu = 0; mu < n; ++mu)
        for (int nu = 0; nu < n; ++nu) {
            const double *A = bs.origin + 3 * mu, *B = bs.origin + 3 * nu;
            const int *a = bs.powers + 3 * mu, *c = bs.powers + 3 * nu;
            double v = 0.0;
            for (int q = 0; q < bs.nprim[nu]; ++q) {
                int pb = bs.prim_off[nu] + q;
                for (int p = 0; p < bs.nprim[mu]; ++p) {
                    int pa = bs.prim_off[mu] + p;
                    v += bs.coefs[pa] * bs.coefs[pb] * bs.norms[pa] * bs.norms[pb] *
                         oq_moment(bs.exps[pa], a[0], a[1], a[2], A[0], A[1], A[2], bs.exps[pb], c[0], c[1], c[2],
                                   B[0], B[1], B[2], C[0], C[1], C[2], ox, oy, oz);
                }
            }
            out[mu * n + nu] = v;
        }
}

/* JK_direct, basis.rs:383-428: every (mu,nu,lambda,sigma), every primitive
 * quartet, the ERI evaluated twice (once for J, once for K).  Rows mu in
 * [mu_begin, mu_end) only, so a bounded sample can be timed; J and K rows in
 * that range are overwritten.  The outer mu loop is split over OpenMP threads
 * when built with -fopenmp (each thread owns whole rows: no reduction). */
void oq_jk_direct(OQ_BASIS_ARGS, void *eri, const double *D, double *J, double *K, int mu_begin, int mu_end) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
#pragma omp parallel for schedule(dynamic, 1)
    for (int mu = mu_begin; mu < mu_end; ++mu) {
        for (int nu = 0; nu < n; ++nu) {
            double jrow = 0.0, krow = 0.0;
            for (int la = 0; la < n; ++la)
                for (int sg = 0; sg < n; ++sg) {
                    double jc = 0.0, kc = 0.0, dls = D[la * n + sg];
                    for (int a = 0; a < bs.nprim[mu]; ++a) {
                        int pa = bs.prim_off[mu] + a;
                        for (int b2 = 0; b2 < bs.nprim[nu]; ++b2) {
                            int pb = bs.prim_off[nu] + b2;
                            for (int c = 0; c < bs.nprim[la]; ++c) {
                                int pc = bs.prim_off[la] + c;
                                for (int d = 0; d < bs.nprim[sg]; ++d) {
                                    int pd = bs.prim_off[sg] + d;
                                    double cc = bs.coefs[pa] * bs.coefs[pb] * bs.coefs[pc] * bs.coefs[pd];
                                    jc += cc * prim_eri(f, &bs, mu, pa, nu, pb, la, pc, sg, pd) * dls;
                                    kc += cc * prim_eri(f, &bs, mu, pa, la, pc, nu, pb, sg, pd) * dls;
                                }
                            }
                        }
                    }
                    jrow += jc;
                    krow += kc;
                }
            J[mu * n + nu] = jrow;
            K[mu * n + nu] = krow;
        }
    }
}

/* build_I, basis.rs:430-460: dense n^4 tensor, 4-fold fill. */
void oq_build_I(OQ_BASIS_ARGS, void *eri, double *I) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
    size_t n2 = (size_t)n * n, n3 = n2 * n;
#pragma omp parallel for schedule(dynamic, 1)
    for (int mu = 0; mu < n; ++mu)
        for (int nu = 0; nu <= mu; ++nu)
            for (int la = 0; la < n; ++la)
                for (int sg = 0; sg <= la; ++sg) {
                    double v = contr_eri(f, &bs, mu, nu, la, sg);
                    I[mu * n3 + nu * n2 + la * (size_t)n + sg] = v;
                    I[nu * n3 + mu * n2 + la * (size_t)n + sg] = v;
                    I[mu * n3 + nu * n2 + sg * (size_t)n + la] = v;
                    I[nu * n3 + mu * n2 + sg * (size_t)n + la] = v;
                }
}

/* JK_inmem, basis.rs:462-484 */
void oq_jk_inmem(int n, const double *I, const double *D, double *J, double *K) {
    size_t n2 = (size_t)n * n, n3 = n2 * n;
    for (int mu = 0; mu < n; ++mu)
        for (int nu = 0; nu <= mu; ++nu) {
            double jc = 0.0, kc = 0.0;
            for (int la = 0; la < n; ++la)
                for (int sg = 0; sg < n; ++sg) {
                    jc += I[mu * n3 + nu * n2 + la * (size_t)n + sg] * D[la * n + sg];
                    kc += I[mu * n3 + la * n2 + nu * (size_t)n + sg] * D[la * n + sg];
                }
            J[mu * n + nu] = J[nu * n + mu] = jc;
            K[mu * n + nu] = K[nu * n + mu] = kc;
        }
}

/* J and K with the same definitions as JK_direct (J_mn = sum (mn|ls) D_ls,
 * K_mn = sum (ml|ns) D_ls) but each unique contracted integral evaluated once
 * (8-fold permutational symmetry, no screening).  D must be symmetric. */
void oq_jk_sym(OQ_BASIS_ARGS, void *eri, const double *D, double *J, double *K) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
    size_t nn = (size_t)n * n;
    long npair = (long)n * (n + 1) / 2;
    int nthr = 1;
#ifdef _OPENMP
    nthr = omp_get_max_threads();
#endif
    double *acc = (double *)calloc((size_t)nthr * 2 * nn, sizeof(double));
#pragma omp parallel for schedule(dynamic, 1)
    for (long ij = 0; ij < npair; ++ij) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *Jt = acc + (size_t)tid * 2 * nn, *Kt = Jt + nn;
        int i = (int)((sqrt(8.0 * ij + 1.0) - 1.0) / 2.0);
        while ((long)i * (i + 1) / 2 > ij) --i;
        while ((long)(i + 1) * (i + 2) / 2 <= ij) ++i;
        int j = (int)(ij - (long)i * (i + 1) / 2);
        for (long kl = 0; kl <= ij; ++kl) {
            int k = (int)((sqrt(8.0 * kl + 1.0) - 1.0) / 2.0);
            while ((long)k * (k + 1) / 2 > kl) --k;
            while ((long)(k + 1) * (k + 2) / 2 <= kl) ++k;
            int l = (int)(kl - (long)k * (k + 1) / 2);
            double v = contr_eri(f, &bs, i, j, k, l);
            if (i == j) v *= 0.5;
            if (k == l) v *= 0.5;
            if (ij == kl) v *= 0.5;
            Jt[i * n + j] += 2.0 * v * D[k * n + l];
            Jt[k * n + l] += 2.0 * v * D[i * n + j];
            Kt[i * n + k] += v * D[j * n + l];
            Kt[j * n + k] += v * D[i * n + l];
            Kt[i * n + l] += v * D[j * n + k];
            Kt[j * n + l] += v * D[i * n + k];
        }
    }
    for (size_t x = 0; x < nn; ++x) { J[x] = 0.0; K[x] = 0.0; }
    for (int t = 0; t < nthr; ++t) {
        double *Jt = acc + (size_t)t * 2 * nn, *Kt = Jt + nn;
        for (size_t x = 0; x < nn; ++x) { J[x] += Jt[x]; K[x] += Kt[x]; }
    }
    free(acc);
    /* symmetrise: J = Jhat + Jhat^T, K = Khat + Khat^T */
    for (int a = 0; a < n; ++a)
        for (int b = 0; b <= a; ++b) {
            double js = J[a * n + b] + J[b * n + a], ks = K[a * n + b] + K[b * n + a];
            J[a * n + b] = J[b * n + a] = js;
            K[a * n + b] = K[b * n + a] = ks;
        }
}

/* pair index ij = i (i + 1) / 2 + j (j <= i) -> (i, j) */
static void pair_of(long ij, int *i, int *j) {
    int a = (int)((sqrt(8.0 * ij + 1.0) - 1.0) / 2.0);
    while ((long)a * (a + 1) / 2 > ij) --a;
    while ((long)(a + 1) * (a + 2) / 2 <= ij) ++a;
    *i = a;
    *j = (int)(ij - (long)a * (a + 1) / 2);
}

/* Schwarz bounds over contracted functions: Q[ij] = sqrt(|(ij|ij)|), so that
 * |(ij|kl)| <= Q[ij] Q[kl].  OpenMP over the pairs. */
void oq_schwarz(OQ_BASIS_ARGS, void *eri, double *Q) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
    long npair = (long)n * (n + 1) / 2;
#pragma omp parallel for schedule(dynamic, 4)
    for (long ij = 0; ij < npair; ++ij) {
        int i, j;
        pair_of(ij, &i, &j);
        Q[ij] = sqrt(fabs(contr_eri(f, &bs, i, j, i, j)));
    }
}

/* oq_jk_sym as a CPU direct-SCF code runs it: each unique contracted integral
 * once, and a quartet skipped when Q[ij] Q[kl] < tau (tau <= 0: no
 * screening).  Only the bra pairs listed in ijs[0..nij) are processed (ijs
 * NULL: all of them, the whole build); a strided subset is a bounded sample
 * of the build.  J and K receive that subset's contributions, symmetrised as
 * in oq_jk_sym.  nthreads > 0 fixes the OpenMP team size (0: all threads).
 * count_only != 0 evaluates nothing and leaves J and K untouched.  Returns
 * the number of contracted integrals that pass the screen. */
long long oq_jk_sym_screened(OQ_BASIS_ARGS, void *eri, const double *D, const double *Q, double tau,
                             const long *ijs, long nij, int nthreads, int count_only, double *J, double *K) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
    size_t nn = (size_t)n * n;
    long npair = (long)n * (n + 1) / 2;
    long nb = ijs ? nij : npair;
    int nthr = 1;
#ifdef _OPENMP
    nthr = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
    double *acc = count_only ? NULL : (double *)calloc((size_t)nthr * 2 * nn, sizeof(double));
    long long count = 0;
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 1) reduction(+ : count)
    for (long t = 0; t < nb; ++t) {
        const long ij = ijs ? ijs[t] : t;
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        int i, j;
        pair_of(ij, &i, &j);
        for (long kl = 0; kl <= ij; ++kl) {
            if (tau > 0.0 && Q[ij] * Q[kl] < tau) continue;
            ++count;
            if (count_only) continue;
            double *Jt = acc + (size_t)tid * 2 * nn, *Kt = Jt + nn;
            int k, l;
            pair_of(kl, &k, &l);
            double v = contr_eri(f, &bs, i, j, k, l);
            if (i == j) v *= 0.5;
            if (k == l) v *= 0.5;
            if (ij == kl) v *= 0.5;
            Jt[i * n + j] += 2.0 * v * D[k * n + l];
            Jt[k * n + l] += 2.0 * v * D[i * n + j];
            Kt[i * n + k] += v * D[j * n + l];
            Kt[j * n + k] += v * D[i * n + l];
            Kt[i * n + l] += v * D[j * n + k];
            Kt[j * n + l] += v * D[i * n + k];
        }
    }
    if (count_only) return count;
    for (size_t x = 0; x < nn; ++x) { J[x] = 0.0; K[x] = 0.0; }
    for (int t = 0; t < nthr; ++t) {
        double *Jt = acc + (size_t)t * 2 * nn, *Kt = Jt + nn;
        for (size_t x = 0; x < nn; ++x) { J[x] += Jt[x]; K[x] += Kt[x]; }
    }
    free(acc);
    for (int a = 0; a < n; ++a)
        for (int b = 0; b <= a; ++b) {
            double js = J[a * n + b] + J[b * n + a], ks = K[a * n + b] + K[b * n + a];
            J[a * n + b] = J[b * n + a] = js;
            K[a * n + b] = K[b * n + a] = ks;
        }
    return count;
}

/* Selected elements J_mn and K_mn, straight from the definitions of
 * basis.rs:406-417 but with contracted integrals (one evaluation per
 * contracted (mn|ls) and (ml|ns)).  For checking full-size Fock builds. */
void oq_jk_elements(OQ_BASIS_ARGS, void *eri, const double *D, int m, const int *mus, const int *nus,
                    double *Jout, double *Kout) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
    for (int e = 0; e < m; ++e) {
        int mu = mus[e], nu = nus[e];
        double jv = 0.0, kv = 0.0;
#pragma omp parallel for reduction(+ : jv, kv) schedule(dynamic, 1)
        for (int la = 0; la < n; ++la)
            for (int sg = 0; sg < n; ++sg) {
                double dls = D[la * n + sg];
                if (sg <= la) {
                    double w = (sg == la) ? 1.0 : 2.0;
                    jv += w * contr_eri(f, &bs, mu, nu, la, sg) * dls;
                }
                kv += contr_eri(f, &bs, mu, la, nu, sg) * dls;
            }
        Jout[e] = jv;
        Kout[e] = kv;
    }
}

int oq_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Elements J_mn, K_mn computed exactly as JK_direct computes them
 * (basis.rs:392-425): for every (lambda, sigma) and every primitive quartet,
 * two primitive ERIs, one for J and one for K.  OpenMP over the elements.
 * Used to time the reference's algorithm on a bounded sample of a Fock build:
 * a full build is n^2 such elements. */
void oq_jk_direct_elements(OQ_BASIS_ARGS, void *eri, const double *D, int m, const int *mus, const int *nus,
                           double *Jout, double *Kout) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
#pragma omp parallel for schedule(dynamic, 1)
    for (int e = 0; e < m; ++e) {
        const int mu = mus[e], nu = nus[e];
        double jv = 0.0, kv = 0.0;
        for (int la = 0; la < n; ++la)
            for (int sg = 0; sg < n; ++sg) {
                double jc = 0.0, kc = 0.0, dls = D[la * n + sg];
                for (int a = 0; a < bs.nprim[mu]; ++a) {
                    int pa = bs.prim_off[mu] + a;
                    for (int b2 = 0; b2 < bs.nprim[nu]; ++b2) {
                        int pb = bs.prim_off[nu] + b2;
                        for (int c = 0; c < bs.nprim[la]; ++c) {
                            int pc = bs.prim_off[la] + c;
                            for (int d = 0; d < bs.nprim[sg]; ++d) {
                                int pd = bs.prim_off[sg] + d;
                                double cc = bs.coefs[pa] * bs.coefs[pb] * bs.coefs[pc] * bs.coefs[pd];
                                jc += cc * prim_eri(f, &bs, mu, pa, nu, pb, la, pc, sg, pd) * dls;
                                kc += cc * prim_eri(f, &bs, mu, pa, la, pc, nu, pb, sg, pd) * dls;
                            }
                        }
                    }
                }
                jv += jc;
                kv += kc;
            }
        Jout[e] = jv;
        Kout[e] = kv;
    }
}

/* The innermost block of JK_direct (basis.rs:400-421) for sampled index
 * quadruples (mu, nu, lambda, sigma): every primitive quartet, two primitive
 * ERIs (one for J, one for K), each weighted by D[lambda][sigma].  A Fock
 * build by the reference's loops is the sum of these blocks over all n^4
 * quadruples, so the mean time per sampled block times n^4 is the time of a
 * whole build.  OpenMP over the samples. */
void oq_jk_direct_quartets(OQ_BASIS_ARGS, void *eri, const double *D, int m, const int *mus, const int *nus,
                           const int *las, const int *sgs, double *Jout, double *Kout) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
#pragma omp parallel for schedule(dynamic, 16)
    for (int e = 0; e < m; ++e) {
        const int mu = mus[e], nu = nus[e], la = las[e], sg = sgs[e];
        const double dls = D[la * n + sg];
        double jc = 0.0, kc = 0.0;
        for (int a = 0; a < bs.nprim[mu]; ++a) {
            int pa = bs.prim_off[mu] + a;
            for (int b2 = 0; b2 < bs.nprim[nu]; ++b2) {
                int pb = bs.prim_off[nu] + b2;
                for (int c = 0; c < bs.nprim[la]; ++c) {
                    int pc = bs.prim_off[la] + c;
                    for (int d = 0; d < bs.nprim[sg]; ++d) {
                        int pd = bs.prim_off[sg] + d;
                        double cc = bs.coefs[pa] * bs.coefs[pb] * bs.coefs[pc] * bs.coefs[pd];
                        jc += cc * prim_eri(f, &bs, mu, pa, nu, pb, la, pc, sg, pd) * dls;
                        kc += cc * prim_eri(f, &bs, mu, pa, la, pc, nu, pb, sg, pd) * dls;
                    }
                }
            }
        }
        Jout[e] = jc;
        Kout[e] = kc;
    }
}

static long pair_idx(int i, int j) { return i >= j ? (long)i * (i + 1) / 2 + j : (long)j * (j + 1) / 2 + i; }

/* Elements J_mn and K_mn as oq_jk_elements, but a contracted integral
 * (ab|cd) is skipped when Q[ab] Q[cd] < tau (Q from oq_schwarz); tau far
 * below the Fock build's threshold keeps the elements exact to well under
 * that threshold while skipping the integrals of distant pairs.  OpenMP over
 * the elements. */
void oq_jk_elements_screened(OQ_BASIS_ARGS, void *eri, const double *D, const double *Q, double tau, int m,
                             const int *mus, const int *nus, double *Jout, double *Kout) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
#pragma omp parallel for schedule(dynamic, 1)
    for (int e = 0; e < m; ++e) {
        const int mu = mus[e], nu = nus[e];
        const double qmn = Q[pair_idx(mu, nu)];
        double jv = 0.0, kv = 0.0;
        for (int la = 0; la < n; ++la) {
            const double qml = Q[pair_idx(mu, la)];
            for (int sg = 0; sg < n; ++sg) {
                const double dls = D[la * n + sg];
                if (sg <= la && qmn * Q[pair_idx(la, sg)] >= tau) {
                    double w = (sg == la) ? 1.0 : 2.0;
                    jv += w * contr_eri(f, &bs, mu, nu, la, sg) * dls;
                }
                if (qml * Q[pair_idx(nu, sg)] >= tau) kv += contr_eri(f, &bs, mu, la, nu, sg) * dls;
            }
        }
        Jout[e] = jv;
        Kout[e] = kv;
    }
}

/* The ERI tensor in the 8-fold packed layout of cints.c:375-387
 * (I[pair(pair(i,j), pair(k,l))] = (ij|kl)), each unique contracted integral
 * once; integrals with Q[ij] Q[kl] < tau are stored as 0 (tau <= 0: none).
 * OpenMP over the bra pairs. */
void oq_eri_packed(OQ_BASIS_ARGS, void *eri, const double *Q, double tau, double *I) {
    OQ_BASIS_INIT;
    oq_eri_fn f = eri ? (oq_eri_fn)eri : oq_coulomb_repulsion;
    long npair = (long)n * (n + 1) / 2;
#pragma omp parallel for schedule(dynamic, 1)
    for (long ij = 0; ij < npair; ++ij) {
        int i, j;
        pair_of(ij, &i, &j);
        double *row = I + (size_t)ij * (ij + 1) / 2;
        for (long kl = 0; kl <= ij; ++kl) {
            if (tau > 0.0 && Q[ij] * Q[kl] < tau) {
                row[kl] = 0.0;
                continue;
            }
            int k, l;
            pair_of(kl, &k, &l);
            row[kl] = contr_eri(f, &bs, i, j, k, l);
        }
    }
}

/* J and K (JK_inmem's definitions, basis.rs:462-484) from the packed tensor
 * of oq_eri_packed: every unique integral scattered to its symmetric
 * positions with the degeneracy weights of oq_jk_sym.  D symmetric. */
void oq_jk_packed(int n, const double *I, const double *D, double *J, double *K) {
    size_t nn = (size_t)n * n;
    long npair = (long)n * (n + 1) / 2;
    int nthr = 1;
#ifdef _OPENMP
    nthr = omp_get_max_threads();
#endif
    double *acc = (double *)calloc((size_t)nthr * 2 * nn, sizeof(double));
#pragma omp parallel for schedule(dynamic, 16)
    for (long ij = 0; ij < npair; ++ij) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *Jt = acc + (size_t)tid * 2 * nn, *Kt = Jt + nn;
        int i, j;
        pair_of(ij, &i, &j);
        const double *row = I + (size_t)ij * (ij + 1) / 2;
        for (long kl = 0; kl <= ij; ++kl) {
            double v = row[kl];
            if (v == 0.0) continue;
            int k, l;
            pair_of(kl, &k, &l);
            if (i == j) v *= 0.5;
            if (k == l) v *= 0.5;
            if (ij == kl) v *= 0.5;
            Jt[i * n + j] += 2.0 * v * D[k * n + l];
            Jt[k * n + l] += 2.0 * v * D[i * n + j];
            Kt[i * n + k] += v * D[j * n + l];
            Kt[j * n + k] += v * D[i * n + l];
            Kt[i * n + l] += v * D[j * n + k];
            Kt[j * n + l] += v * D[i * n + k];
        }
    }
    for (size_t x = 0; x < nn; ++x) { J[x] = 0.0; K[x] = 0.0; }
    for (int t = 0; t < nthr; ++t) {
        double *Jt = acc + (size_t)t * 2 * nn, *Kt = Jt + nn;
        for (size_t x = 0; x < nn; ++x) { J[x] += Jt[x]; K[x] += Kt[x]; }
    }
    free(acc);
    for (int a = 0; a < n; ++a)
        for (int b = 0; b <= a; ++b) {
            double js = J[a * n + b] + J[b * n + a], ks = K[a * n + b] + K[b * n + a];
            J[a * n + b] = J[b * n + a] = js;
            K[a * n + b] = K[b * n + a] = ks;
        }
}
