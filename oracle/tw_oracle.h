/*
 * tw_oracle.h -- CPU oracle for the TetWild mesh-optimisation query path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GB300
 * kernels are compared against.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it; the product library
 * (tetwild_gb300/libtw_gb300.so) never links or calls it.
 *
 * Every routine restates one reference routine (TetWild, file:line given at
 * each function) in plain C99.  The arithmetic of each routine is written out
 * operation by operation, in the same order as the CUDA device code in
 * tetwild_gb300/csrc/, so that results are bit-identical when both sides are
 * built without FP contraction (host: -ffp-contract=off, device: -fmad=false).
 *
 * Pinning: the AMIPS energy/gradient/Hessian are checked against the
 * reference's own generated expressions (compiled from the reference sources
 * into oracle/_ref by oracle/ref/build_ref.py); orientation and collinearity
 * signs are checked against exact rational arithmetic (Python fractions);
 * sampleTriangle and the envelope traversal are checked against the
 * reference's sampleTriangle / MeshFacetsAABBWithEps compiled into oracle/_ref.
 */
#ifndef TW_ORACLE_H
#define TW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- AMIPS (LocalOperations.cpp:28-291) ---------------------------------- */
double two_icbrt(double x);                                   /* x^(-1/3)      */
/* The unsuffixed routines evaluate the selected form: TWO_FORM_REFERENCE
 * (default) performs the reference's generated operations in its order and
 * agrees with it to its rounding; TWO_FORM_CLOSED is the accurate closed
 * form.  The selection is process-wide; set it before a batch call.         */
#define TWO_FORM_REFERENCE 0
#define TWO_FORM_CLOSED 1
void   two_set_energy_form(int form);
int    two_get_energy_form(void);
double two_amips_energy(const double T[12]);                  /* :28-81        */
void   two_amips_jacobian(const double T[12], double J[3]);   /* :83-147       */
void   two_amips_hessian(const double T[12], double H[9]);    /* :149-291      */
double two_amips_energy_rf(const double T[12]);
void   two_amips_jacobian_rf(const double T[12], double J[3]);
void   two_amips_hessian_rf(const double T[12], double H[9]);
double two_amips_energy_cf(const double T[12]);
void   two_amips_jacobian_cf(const double T[12], double J[3]);
void   two_amips_hessian_cf(const double T[12], double H[9]);
double two_rf_pow_m13(double s);                 /* s^-0.333333333333333 */

/* ---- exact predicates (CGAL Epick orientation / collinear) --------------- */
/* +1 POSITIVE, 0 COPLANAR, -1 NEGATIVE; CGAL convention:
 * sign(det[q-p, r-p, s-p]).  Non-finite input returns 0.                    */
int two_orient3d(const double p[3], const double q[3], const double r[3], const double s[3]);
int two_orient3d_exact(const double p[3], const double q[3], const double r[3], const double s[3]);
int two_collinear(const double a[3], const double b[3], const double c[3]);

/* ---- tet quality (LocalOperations.cpp:695-773, :862-884) ----------------- */
#define TWO_MAX_ENERGY 1e50
/* calTetQuality_AMIPS: orientation != POSITIVE, inf, nan or <= 0 -> 1e50.   */
double two_tet_quality(const double T[12]);
/* isTetFlip on rounded coordinates (:535-553): 1 if orientation != POSITIVE */
int two_tet_flip(const double T[12]);

/* ---- distances ------------------------------------------------------------ */
double two_point_triangle_sqdist(const double p[3], const double a[3], const double b[3],
                                 const double c[3], double q[3]);
double two_point_box_sqdist(const double p[3], const double lo[3], const double hi[3]);

/* ---- sampleTriangle (Common.cpp:143-228) ---------------------------------- */
/* Writes up to cap samples (xyz) into out; returns the full sample count
 * (may exceed cap, in which case only the first cap were written).          */
int64_t two_sample_triangle(const double v[9], double sampling_dist, double* out, int64_t cap);
/* Only the count (same rules, no writes).                                   */
int64_t two_sample_count(const double v[9], double sampling_dist);

/* ---- envelope (LocalOperations.cpp:1034-1109, mesh_AABB.cpp:418-548) ------ */
typedef struct two_surface two_surface;
two_surface* two_surface_build(const double* V, int32_t nV, const int32_t* F, int32_t nF);
void         two_surface_free(two_surface* s);
/* isPointOutEnvelop: 1 iff every facet f has sqdist(p, f) > eps2.           */
int two_point_out(const two_surface* s, const double p[3], double eps2);
/* Brute force over all facets (test of the tree): same decision.            */
int two_point_out_brute(const two_surface* s, const double p[3], double eps2);
/* isFaceOutEnvelop_sampling: degenerate -> 0; else 1 iff a sample is out.   */
int two_face_out(const two_surface* s, const double tri[9], double eps2, double sampling_dist);

/* ---- Newton smoothing of one star (VertexSmoother.cpp:465-702) ----------- */
/* 3x3 solve by Householder QR with column pivoting.  Returns 0 on success.  */
int two_qr_solve3(const double H[9], const double b[3], double x[3]);
/* NewtonsMethod for one star.  xyz: vertex coordinates (AoS, all vertices
 * referenced by tets), tets: 4 ids per tet in caller order, v: centre id.
 * Writes the new position to out[3]; returns is_moved (0/1).                */
int two_newton_star(const double* xyz, const int32_t* tets, int32_t ntets, int32_t v,
                    int max_step, int max_it, double out[3]);

/* ---- nearest facet (MeshFacetsAABBWithEps::nearest_facet, mesh_AABB.h:130) */
/* Returns the input index of the nearest facet (smallest squared distance,  *
 * ties to the smallest index), its closest point q and the squared distance.*/
int32_t two_nearest_facet(const two_surface* s, const double p[3], double q[3], double* sqd);
int32_t two_nearest_facet_brute(const two_surface* s, const double p[3], double q[3], double* sqd);

/* ---- one vertex of a smoothing pass (VertexSmoother.cpp:114-210, 244-450) - */
#define TWO_STAR_INTERIOR 0
#define TWO_STAR_SURFACE 1
#define TWO_STAR_BOUNDARY 2
#define TWO_SMOOTH_INVALID 0
#define TWO_SMOOTH_NOT_MOVED 1
#define TWO_SMOOTH_MOVED 2
#define TWO_SMOOTH_REJECT_FLIP 3
#define TWO_SMOOTH_REJECT_QUALITY 4
#define TWO_SMOOTH_REJECT_ENVELOPE 5
int two_smooth_star(const double* xyz, const int32_t* tets, const uint8_t* fflags, int32_t ntets,
                    int32_t v, int kind, const two_surface* s_in, const two_surface* s_b,
                    double eps2, double sampling_dist, int max_step, int max_it, double out[3]);

/* ---- checks of one edge collapse (EdgeCollapser.cpp:284-446, :727-775) --- */
#define TWO_CV_V1_SURFACE 1
#define TWO_CV_V1_BOUNDARY 2
#define TWO_CV_V2_SURFACE 4
#define TWO_CV_V2_BOUNDARY 8
#define TWO_CV_V1_UNROUNDED 16
int two_collapse_check(const double* xyz, const int32_t* tets, const uint8_t* fflags, int32_t ntets,
                       int32_t v1, int32_t v2, int flags, const two_surface* s_in,
                       const two_surface* s_b, double eps2, double sampling_dist,
                       int check_quality, double soft_energy);

/* ---- energy sweeps (LocalOperations.cpp:605-693) ------------------------- */
/* calTetQuality_AD (LocalOperations.cpp:783-860): the smallest and largest
 * dihedral angle of tet T, (0, pi) for a degenerate one. */
void two_dihedral_minmax(const double T[12], double* min_angle, double* max_angle);
/* outputInfo's dihedral sweep (LocalOperations.cpp:483-521) over tets not
 * locked: out = {min, sum of mins / cnt, max, sum of maxes / cnt} (sums in tet
 * order), counts = {min < 6, 12, 18 deg, max > 162, 168, 174 deg, cnt};
 * per-tet angles when mins / maxs are non-NULL. */
void two_dihedral_stats(const double* xyz, const int32_t* tets, int64_t n, const uint8_t* locked,
                        double out[4], int64_t counts[7], double* mins, double* maxs);
void two_energy_stats(const double* xyz, const int32_t* tets, int64_t n, const uint8_t* locked,
                      double filter_energy_thres, double* avg, double* max_e,
                      double* second_max, int64_t buckets[11]);
double two_filter_energy(const int64_t buckets[11], double filter_energy_thres, int* is_clean_up);

/* ---- batch drivers (pthreads; nthreads <= 0 means 1) --------------------- */
/* T is SoA [12][n] (the energy_ispc layout).  Any output may be NULL.       *
 * J and H are SoA ([3][n], [9][n]).  flip[i] = two_tet_flip; E[i] is the    *
 * calTetQualities value when quality!=0, else the raw energy.               */
void two_amips_batch_soa(const double* T, int64_t n, int quality, double* E, double* J,
                         double* H, uint8_t* flip, int nthreads);
void two_points_out_batch(const two_surface* s, const double* P, int64_t n, double eps2,
                          uint8_t* out, int nthreads);
void two_faces_out_batch(const two_surface* s, const double* tris, int64_t n, double eps2,
                         double sampling_dist, uint8_t* out, int nthreads);
void two_newton_stars_batch(const double* xyz, const int32_t* star_off, const int32_t* tets,
                            const int32_t* centers, int64_t nstars, int max_step, int max_it,
                            double* out, uint8_t* moved, int nthreads);

void two_smooth_stars_batch(const double* xyz, const int32_t* star_off, const int32_t* tets,
                            const uint8_t* fflags, const int32_t* centers, const uint8_t* kinds,
                            int64_t nstars, const two_surface* s_in, const two_surface* s_b,
                            double eps2, double sampling_dist, int max_step, int max_it,
                            double* out, int8_t* status, int nthreads);
void two_nearest_batch(const two_surface* s, const double* P, int64_t n, double* Q, double* D,
                       int32_t* F, int nthreads);
/* ---- edge removal (EdgeRemover.cpp:125-600) ------------------------------ */
int two_swap_check(const double* xyz, const int32_t* shell, int32_t k, int32_t v1, int32_t v2,
                   int budget, int* config, int* spent);
void two_swap_check_batch(const double* xyz, const int32_t* off, const int32_t* tets,
                          const int32_t* v12, const int32_t* budget, int64_t n, uint8_t* result,
                          int8_t* config, uint8_t* spent);
void two_collapse_check_batch(const double* xyz, const int32_t* off, const int32_t* tets,
                              const uint8_t* fflags, const int32_t* v12, const uint8_t* flags,
                              int64_t n, const two_surface* s_in, const two_surface* s_b,
                              double eps2, double sampling_dist, int check_quality,
                              double soft_energy, uint8_t* result, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
