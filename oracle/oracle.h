/*
 * oracle.h -- C interface of the CPU oracle (liboracle.so).
 *
 * TEST INFRASTRUCTURE.  The oracle is a libMesh-free FP64 restatement of the
 * reference's explicit time step (ShellSystem.C) used to check the CUDA
 * library; only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  It is never part of the product path.
 *
 * Functions return 0 on success, a ShellSystem::Problem value (1..7) when a
 * problem was registered, or -1 on a usage error (message in oracle_error()).
 */
#ifndef SHELL_ORACLE_H_
#define SHELL_ORACLE_H_

#include <stddef.h>
#include <stdint.h>
#include "../include/shl.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle oracle;

const char* oracle_error(void);
void oracle_set_threads(int n);

oracle* oracle_create(const shl_mesh* mesh, const shl_params* params);
void oracle_destroy(oracle* o);

int oracle_apply_initial_conditions(oracle* o, const double* u0, double t0, double pressure_next);
int oracle_set_state(oracle* o, const double* u, const double* v, const double* a);
int oracle_get_state(oracle* o, double* u, double* v, double* a);
int oracle_set_time(oracle* o, double t, uint32_t time_step);
int oracle_get_time(oracle* o, double* t, uint32_t* time_step);

int oracle_eval_forces(oracle* o, const double* u_pred, const double* v_pred, double pressure,
                       double* f_out, double* a_out, shl_energies* e);
int oracle_step(oracle* o, uint32_t n_steps, const double* pressure_table, shl_step_report* r);

size_t oracle_get_contact_state(oracle* o, uint32_t* pairs, uint8_t* stick, double* origin,
                                double* d2, size_t cap, double* du_sum);
int oracle_set_contact_state(oracle* o, const uint32_t* pairs, const uint8_t* stick,
                             const double* origin, const double* d2, size_t n, double du_sum);
int oracle_rebuild_contacts(oracle* o);
int oracle_get_mass_damping(oracle* o, double* Minv, double* C);
/* Pressure as a config expression of t (evaluated each attempt); NULL or "" = table. */
int oracle_set_pressure_function(oracle* o, const char* expr);
/* Cavity semi-axes as expressions of t (NULL/"" = the constants of the parameters). */
int oracle_set_cavity_functions(oracle* o, const char* rx, const char* ry, const char* rz);
/* Cavity spring origins (3V), cavity energy densities (V) and (Ecav, cavity force, Nc_cav). */
int oracle_get_cavity(oracle* o, double* origins, double* ecav, double* out3);
/* Current time step size (adaptive dt) and the number of repeated steps so far. */
double oracle_get_dt(oracle* o);
uint64_t oracle_get_rejections(oracle* o);
/* node_vectors ekin, eself, efric of the last step (ShellSystem.C:126-130). */
int oracle_get_node_fields(oracle* o, double* ekin, double* eself, double* efric);
int oracle_get_element_fields(oracle* o, double* kGauss, double* kMean, double* etens,
                              double* ebend, double* area);
/* avg_elem_size, cell_size, d_max and the bounds of the last rebuild */
int oracle_get_cell_info(oracle* o, double* out /* 9 */);

/* ---- known-answer helpers ---- */
/* patch node ids of element eid in the oracle's patch order (up to 12) */
int oracle_patch(oracle* o, uint32_t eid, uint32_t* nodes, uint32_t* n);
/* SMOOTH contact: the minimiser's start / end point (v1, w1, v2, w2) in each
 * face's patch frame, per pair in (eid1, eid2) order */
size_t oracle_get_contact_coords(oracle* o, double* x, size_t cap);
int oracle_set_contact_coords(oracle* o, const double* x, size_t n);
/* SMOOTH: limit surface of face eid at patch-frame (v, w) at the current
 * positions: out[3*k + c], k = point, d/dv, d/dw, d2/dv2, d2/dw2, d2/dvdw */
int oracle_limit_eval(oracle* o, uint32_t eid, double v, double w, double* out);
/* SMOOTH: the same as weights of the patch nodes, out[6*j + k] */
int oracle_limit_basis(oracle* o, uint32_t eid, double v, double w, double* out);
/* SMOOTH: closest points of the limit patches of e1 and e2 from start x[4];
 * returns the iterations, x the minimiser, d2 and dc = p2 - p1 */
int oracle_smooth_closest(oracle* o, uint32_t e1, uint32_t e2, double* x, double* d2, double* dc);
/* subdivision table of valence N (shl_subdiv.h layout); returns its length */
size_t oracle_subdiv_table(int N, double* out, size_t cap);
/* unrotated basis of element eid at element parameters (v, w):
 * out[6*i + k], k = phi, d/dv, d/dw, d2/dv2, d2/dw2, d2/dvdw, in patch order.
 * Regular patches: any (v, w); irregular patches: the middle triangle of the
 * first subdivision (v < 1/2, w < 1/2, v + w > 1/2). */
int oracle_basis_at(oracle* o, uint32_t eid, double v, double w, double* out);
/* rotated basis at the quadrature point as cached (same layout) and R (2x2, row major) */
int oracle_basis_cached(oracle* o, uint32_t eid, double* out, double* R);
/* surface metric: which = 0 reference, 1 deformed: xyz(3) vec(9) dvec(9) ff1(3) ff2(3) jac JxW */
int oracle_elem_metric(oracle* o, uint32_t eid, int which, double* out /* 29 */);
/* close_elems of eid (sorted) */
int oracle_close_elems(oracle* o, uint32_t eid, uint32_t* out, size_t cap, size_t* n);

void oracle_segment_segment(const double* p10, const double* p11, const double* p20,
                            const double* p21, double* diffvec, double* st);
void oracle_point_triangle(const double* p0, const double* p1, const double* p2,
                           const double* p3, double* diffvec, double* vw);
/* p: 18 doubles (3 nodes of element 1, 3 of element 2); out: d2, dc(3), v1, w1, v2, w2 */
void oracle_pair_compute(const double* p, double* out);
void oracle_friction_apply(double* Efric, double* f_contact, double f_normal, const double* n,
                           const double* v, double abs_v_normal, double v_stop, double k,
                           double mu_s, double mu_d, double damping, int* stick,
                           double* spring_origin, const double* contact_point);
double oracle_fixed_order_sum(const double* x, uint32_t n);
/* 1 if this build rounds a*b+c in two steps (built with -ffp-contract=off) */
int oracle_fp_contract_off(void);

#ifdef __cplusplus
}
#endif

#endif
