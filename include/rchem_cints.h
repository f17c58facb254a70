/*
 * rchem_cints.h -- drop-in for the reference's bindgen boundary.
 *
 * The reference's Rust code binds libpyquante2/cints.h with bindgen
 * (build.rs:12-19) and calls it through src/integrals/tho66.rs:225-260.  These
 * entry points have the same names, argument order and meaning as the
 * declarations they replace, so the same bindgen step over this header gives
 * the same Rust signatures; each one evaluates its integral on the GPU
 * (a one-element batch of the batched kernels below) and returns the value.
 * On failure the double-returning functions return NaN and set
 * rchem_last_error().
 *
 * The batched entry points are the ones to use for more than a handful of
 * values: one launch per call.
 */
#ifndef RCHEM_CINTS_H
#define RCHEM_CINTS_H

#ifdef __cplusplus
extern "C" {
#endif

/* cints.h:23-29 -- primitive Cartesian ERI (ab|cd) times norma*normb*normc*normd */
double coulomb_repulsion(double xa, double ya, double za, double norma, int la, int ma, int na, double alphaa,
                         double xb, double yb, double zb, double normb, int lb, int mb, int nb, double alphab,
                         double xc, double yc, double zc, double normc, int lc, int mc, int nc, double alphac,
                         double xd, double yd, double zd, double normd, int ld, int md, int nd, double alphad);

/* cints.h:44-47 -- primitive overlap (unnormalised) */
double overlap(double alpha1, int l1, int m1, int n1, double xa, double ya, double za, double alpha2, int l2,
               int m2, int n2, double xb, double yb, double zb);

/* cints.h:40-43 -- primitive kinetic energy (unnormalised) */
double kinetic(double alpha1, int l1, int m1, int n1, double xa, double ya, double za, double alpha2, int l2,
               int m2, int n2, double xb, double yb, double zb);

/* cints.h:50-54 -- primitive nuclear attraction to a unit charge at (x3,y3,z3),
 * times norm1*norm2, negative sign included */
double nuclear_attraction(double x1, double y1, double z1, double norm1, int l1, int m1, int n1, double alpha1,
                          double x2, double y2, double z2, double norm2, int l2, int m2, int n2, double alpha2,
                          double x3, double y3, double z3);

/* cints.h:72 -- position of (ij|kl) in the 8-fold packed ERI array
 * (rchem_build_I_packed's layout) */
int ijkl2intindex(int i, int j, int k, int l);

/* cints.h:69 -- Boys function F_m(x) (exact to ~1e-15 relative; the reference's
 * NR implementation, cints.c:302-373, is accurate to ~1e-7) */
double Fgamma(double m, double x);

/* cints.h:14-21 -- contracted ERI: sum over primitives of coefs * (ab|cd) with
 * the per-primitive norms */
double contr_coulomb(int ia, double *aexps, double *acoefs, double *anorms, double xa, double ya, double za, int la,
                     int ma, int na, int ib, double *bexps, double *bcoefs, double *bnorms, double xb, double yb,
                     double zb, int lb, int mb, int nb, int ic, double *cexps, double *ccoefs, double *cnorms,
                     double xc, double yc, double zc, int lc, int mc, int nc, int id, double *dexps,
                     double *dcoefs, double *dnorms, double xd, double yd, double zd, int ld, int md, int nd);

/* One primitive Gaussian: centre, norm, exponent, Cartesian powers. */
typedef struct {
    double x, y, z, norm, alpha;
    int l, m, n, pad;
} rchem_prim;

/* out[i] = coulomb_repulsion of quartet i (prims[4i..4i+3]); total L <= 12. */
int rchem_eri_prim_batch(int count, const rchem_prim *prims, double *out, int where);
/* kind 0 = overlap, 1 = kinetic (both unnormalised, pair i = prims[2i..2i+1]),
 * 2 = nuclear_attraction (with norms and sign; centre i = centers[3i..3i+2]). */
int rchem_onee_prim_batch(int kind, int count, const rchem_prim *prims, const double *centers, double *out,
                          int where);
/* out[i] = F_m[i](x[i]); precision 64 (0 <= m <= 16; the run-time-m evaluation
 * of the gradient kernels), 65 (0 <= m <= 8; the branch-free FP64 evaluation of
 * the ERI kernels, through its L = 8 downward recursion) or 32 (the kernels' FP32
 * Boys, widened).  A device-resident m outside the range gives NaN. */
int rchem_boys_batch(int count, const int *m, const double *x, double *out, int precision, int where);

#ifdef __cplusplus
}
#endif
#endif /* RCHEM_CINTS_H */
