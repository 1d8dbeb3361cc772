/* sep_oracle.h -- CPU restatement of the reference separation likelihood.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA path is compared
 * against; it is never linked into, loaded by or called from the product
 * library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg use it.
 *
 * The restatement follows milkyway_separation/cpu/evaluation_optimized.c of
 * the reference operation by operation (same formulas, same association order,
 * same libm calls) so that, compiled with -ffp-contract=off, it reproduces the
 * reference's doubles.  It is pinned against the reference compiled from its
 * own sources (oracle/_ref, oracle/Makefile `ref`) and against the golden
 * values committed under tests/golden/.
 */
#ifndef SEP_ORACLE_H
#define SEP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct so_problem so_problem;

/* Load a parameter file (reference format, cpu/parameters.c:107-228) and a
 * star file (cpu/star_points.c:69-81).  star_path may be NULL (integrals
 * only).  Returns NULL on a parse error. */
so_problem* so_open(const char* param_path, const char* star_path);
void so_close(so_problem* p);

int so_n_theta(const so_problem* p);   /* get_optimized_parameter_count */
int so_n_streams(const so_problem* p);
int so_n_areas(const so_problem* p);
int so_n_stars(const so_problem* p);
int so_convolve(const so_problem* p);
/* area dims: out[0..2] = mu_steps, nu_steps, r_steps */
int so_area_dims(const so_problem* p, int area, int* out);

/* Full evaluation = cpu_evaluate (evaluation_optimized.c:756-784).
 *   rank/nranks: the reference's own slicing of the linearised cell index
 *     and of the catalogue (parameters.c:502-522, star_points.c:105-131);
 *     nranks <= 1 evaluates everything.
 *   area_integrals: (1+S) per area; integrals: (1+S) after the cut
 *     subtraction; likelihood = prob_sum/N - 3.0 (app :278);
 *   bg_only / st_only: the background-only and per-stream-only mean log10
 *     likelihoods (evaluation_optimized.c:719-731, minus 3.0).
 * Any output pointer may be NULL.  Returns 0 on success. */
int so_evaluate(so_problem* p, const double* theta, int rank, int nranks,
                double* area_integrals, double* integrals,
                double* prob_sum, int* num_zero, double* likelihood,
                double* bg_only, double* st_only);

/* Integrals only (no likelihood).  Same conventions as so_evaluate. */
int so_integrals(so_problem* p, const double* theta, int rank, int nranks,
                 double* area_integrals, double* integrals);

/* Likelihood only, with caller-supplied integrals (1+S). */
int so_likelihood(so_problem* p, const double* theta, const double* integrals,
                  double* prob_sum, int* num_zero, double* likelihood,
                  double* bg_only, double* st_only);

/* Per-cell values bg*V and st_s*V of one area, laid out
 * [mu][nu][r][1+S] (the reference's linear order).  For small cases. */
int so_cell_values(so_problem* p, const double* theta, int area, double* out);

/* Per-(mu,nu) Galactic (l, b) in degrees of one area: out[mu][nu][2]. */
int so_cell_lb(so_problem* p, int area, double* out);

/* r-bin tables of one area (cpu__r_constants, :360-422):
 * irv[R], reff_xr_rp3[R], r_point[R][C], qw_r3_N[R][C], ids[Nnu], nus[Nnu]. */
int so_r_tables(so_problem* p, int area, double* irv, double* reff_xr_rp3,
                double* r_point, double* qw_r3_N, double* ids, double* nus);
/* The same area's r_in_mag / r_in_mag2 tables [R][C] (set_probability_constants,
 * cpu/evaluation_optimized.c:159-188), for the aux profile. */
int so_r_mag_tables(so_problem* p, int area, double* r_in_mag, double* r_in_mag2);

/* Per-star unnormalised densities (calculate_probabilities on the star):
 * bg[N], st[N][S]. */
int so_star_densities(so_problem* p, const double* theta, double* bg, double* st);

/* The separation output (milkyway_separation/cpu/separation.c:37-254, a
 * program the reference no longer builds): with integrals (1+S) from an
 * evaluation, per star the stream-membership probabilities
 * sprob[N][S] = psg_s / (sum psg + pbx) (:128-199), and the star's position
 * in the stripe frame xyz[N][3] (:75-116, :226-227).  expected[S] = the
 * sequential sum of sprob over stars (:193-196).  Any output may be NULL. */
int so_separation(so_problem* p, const double* theta, const double* integrals, double* sprob, double* xyz,
                  double* expected);
/* The stripe-frame rotation (stripe_normal or sgr_stripe_normal, then
 * get_transform to the z axis): mat9 row-major. */
void so_stripe_transform(int sgr, int wedge, double* mat9);
/* transform_point (stVector.c:155-169) with the Sun at (-8.5, 0, 0). */
void so_transform_point(const double* xyz, const double* mat9, double* out);

/* Gauss-Legendre nodes/weights on [-1,1] (numericalIntegration.c:67-104). */
void so_gauss_legendre(int n, double* x, double* w);

/* Geometry helpers exposed for known-answer tests. */
void so_gc_to_lb(int wedge, double mu, double nu, double* l, double* b);
void so_lbr_to_xyz(double l, double b, double r, double* xyz);

#ifdef __cplusplus
}
#endif
#endif
