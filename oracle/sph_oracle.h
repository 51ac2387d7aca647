/* CPU restatement ("port") of the reference SPH step, in plain C with OpenMP.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm may load it, and only as the checker or the
 * timed CPU baseline -- never as part of the product path.
 *
 * Parameter blocks are 16 floats in SPHParameters field order (src/sph_engine.h:14-34):
 *   rest_density, gas_constant, viscosity, smoothing_length, particle_mass, timestep,
 *   gravity, damping, CFL_factor, xmin, xmax, ymin, ymax, zmin, zmax,
 *   neighbor_search_radius
 * Vectors are flat float arrays, 3 floats per particle, in insertion order.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Neighbour lists exactly as SpatialHash::query_squared produces them
 * (src/spatial_hash.cpp:31-57): order, self included.  counts[n]; idx (optional) gets the
 * concatenated lists.  Returns the total number of entries. */
int64_t orc_query(size_t n, const float* pos, float cell_size, float radius, int64_t* counts,
                  int64_t* idx);

/* The lists of the particles sel[0..nq) (insertion indices) among all n particles, as
 * orc_query gives them, without building the other particles' lists.  Returns the total
 * number of entries; counts[nq]; idx (optional) gets the concatenated lists. */
int64_t orc_query_subset(size_t n, const float* pos, float cell_size, float radius, size_t nq,
                         const int64_t* sel, int64_t* counts, int64_t* idx);

/* One evaluation of density, pressure and acceleration on a given state, in FP32 with the
 * reference's operation order (src/sph_engine.cpp:203-244, 370-443). */
void orc_fields(size_t n, const float* pos, const float* vel, const float* mass,
                const float* params16, float* rho, float* P, float* acc);

/* orc_fields with the smoothing kernel `kind` of create_kernel (src/kernels.cpp:226-236):
 * 0 CUBIC_SPLINE, 1 WENDLAND_C2, 2 GAUSSIAN, evaluated through the equations:: formulas
 * (the reference engine itself always uses the cubic spline, sph_engine.cpp:17, 23, 162). */
void orc_fields_k(int kind, size_t n, const float* pos, const float* vel, const float* mass,
                  const float* params16, float* rho, float* P, float* acc);

/* The same evaluation in FP64 over the same (FP32-defined) neighbour sets: the
 * high-precision reference for error figures.  Optionally (sum_abs != NULL) also returns,
 * per particle and component, the sum of |term| of the acceleration's pair terms divided
 * by m_i: the conditioning scale against which FP32 force errors are judged. */
void orc_fields_f64(size_t n, const float* pos, const float* vel, const float* mass,
                    const float* params16, double* rho, double* P, double* acc,
                    double* sum_abs);

void orc_fields_f64_k(int kind, size_t n, const float* pos, const float* vel,
                      const float* mass, const float* params16, double* rho, double* P,
                      double* acc, double* sum_abs);

/* FP64 evaluation on FP64 positions (the truth for the precision study): neighbour sets
 * by dot(x_i - x_j, x_i - x_j) <= r^2 in double, density/pressure/acceleration in double
 * with the reference's formulas.  Returns the total number of (i, j) pairs. */
int64_t orc_fields_f64d(size_t n, const double* pos, const float* vel, const float* mass,
                        const float* params16, double* rho, double* P, double* acc);
/* orc_fields_f64d plus, when sum_abs != NULL, the per-component sum of |term| / m of each
 * acceleration (the conditioning scale of orc_fields_f64). */
int64_t orc_fields_f64d_s(size_t n, const double* pos, const float* vel, const float* mass,
                          const float* params16, double* rho, double* P, double* acc,
                          double* sum_abs);

/* ---- engine: restatement of SPHEngine state and step (src/sph_engine.cpp:13-353) ---- */
typedef struct orc_engine orc_engine;
orc_engine* orc_engine_new(size_t capacity);
void orc_engine_free(orc_engine* e);
void orc_engine_initialize(orc_engine* e, const float* params16);
/* Smoothing kernel of the engine's step (kind as in orc_fields_k; default 0). */
void orc_engine_set_kernel(orc_engine* e, int kind);
/* Appends particles; beyond capacity they are dropped (src/particle.cpp:26-33).
 * vel may be NULL (zero velocity). */
void orc_engine_add(orc_engine* e, size_t n, const float* pos, const float* vel,
                    const float* mass);
void orc_engine_clear(orc_engine* e);
void orc_engine_step(orc_engine* e, float dt);
size_t orc_engine_size(const orc_engine* e);
float orc_engine_time(const orc_engine* e);
uint64_t orc_engine_step_count(const orc_engine* e);
/* pos/vel/acc: 3*size floats (acc = the engine's accelerations_ buffer);
 * rho/P: capacity floats (get_densities()/get_pressures()). Any pointer may be NULL. */
void orc_engine_get(const orc_engine* e, float* pos, float* vel, float* acc, float* rho,
                    float* P);
/* Overwrites the state of the first size() particles (pos/vel may be NULL). */
void orc_engine_set_state(orc_engine* e, const float* pos, const float* vel);
/* total_mass, total_energy, mass_error, energy_error, max_neighbors,
 * total_neighbor_queries (src/sph_engine.cpp:178-200). */
void orc_engine_diag(const orc_engine* e, double* out6);
/* Last CFL timestep the engine computed (0 if none). */
float orc_engine_last_dt(const orc_engine* e);

int orc_max_threads(void);
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
