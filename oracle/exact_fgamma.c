/*
 * exact_fgamma.c -- CPU ORACLE (test infrastructure only).
 *
 * A strong definition of the reference's Boys entry point
 * (libpyquante2/cints.h: double Fgamma(double m, double x)) that evaluates
 * F_m(x) exactly (oq_boys_exact in pq2_port.c).  build_ref.mk links it
 * beside the reference's own cints.o/chgp.o, whose Fgamma has been made weak,
 * so every internal Boys call of the unmodified reference integrals binds
 * here.  Result: the reference's THO integrals with a ~1e-16 Boys function,
 * the 1e-12-per-integral parity oracle.
 */
double oq_boys_exact(int m, double x);

double Fgamma(double m, double x) { return oq_boys_exact((int)(m + 0.5), x); }
