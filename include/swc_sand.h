/*
 * swc_sand.h -- C ABI of the GB300 DEM sand step.  Drop-in for
 * DEMParticleSand<Dim>::advance of skytang0205/sand-water-coupling
 * (Cores/Physics/DEMParticleSand.h:13-58, DEMParticleSand.cpp:90-152) with the
 * contact model of DEMParticle (Cores/Structures/DEMParticle.h:57-112,
 * DEMParticle.cpp:15-134).
 *
 * Conventions (as include/swc.h)
 *   - One context owns every device buffer of one sand simulation on one GPU
 *     and one CUDA stream.  Calls on a context are not re-entrant.
 *   - Host arrays are FP64, `dim` components per particle, particle-major (the
 *     .sav layout, Cores/Utilities/IO.h:19-26); they are copied, never retained.
 *   - Device positions are float-float pairs (about 48 significant bits): the
 *     contact law acts on penetration depths of ~1e-6 r at rest, far below
 *     FP32's resolution of absolute positions.  Velocities and forces are FP32.
 *   - Every call returns an swc_status code (include/swc.h).  There is no CPU
 *     fallback: without a usable GPU swc_sand_create fails with SWC_CUDA_ERROR.
 *   - The reference updates velocities[i] in a parallel loop that reads the
 *     velocities of neighbours (DEMParticleSand.cpp:130-151), so its result
 *     depends on thread timing.  Here every particle of one step reads the
 *     velocities from the start of the contact pass.
 */
#ifndef SWC_SAND_H
#define SWC_SAND_H

#include <stddef.h>
#include <stdint.h>

#include "swc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct swc_sand swc_sand;

/* Replaces the constructor DEMParticleSand(particleRadius) and the DEMParticle
 * setters (DEMParticle.cpp:15-60). */
typedef struct swc_sand_params {
    int32_t dim;            /* 2 or 3 */
    int32_t enable_gravity; /* DEMParticleSand::_enableGravity (true in the reference) */
    double  radius;         /* particle radius r: contacts at |d| < 2r, boundary reach 4r */
    double  mass;           /* particle mass (and boundary mass, DEMParticleSand.cpp:79) */
    double  young;          /* DEMParticle::setYoung; K_norm = young * r (default 1e9) */
    double  poisson;        /* DEMParticle::setPoisson; K_tang = K_norm * poisson (default 0.3) */
    double  fric_angle;     /* DEMParticle::setfricangle, radians; tan is taken (default 0.5) */
} swc_sand_params;

/* Reference defaults: gravity on, young 1e9, poisson 0.3, friction angle 0.5 rad, mass 1. */
void swc_sand_default_params(swc_sand_params * p);
const char * swc_sand_last_error(const swc_sand * s);

int  swc_sand_create(const swc_sand_params * p, swc_sand ** out);
void swc_sand_destroy(swc_sand * s);
/* Run on a caller's stream (NULL: the context's own). */
int swc_sand_set_stream(swc_sand * s, void * stream);

/* Particle state (DEMParticleSand::addShape DEMParticleSand.cpp:167-175 for a fresh
 * context, loadFrame DEMParticleSand.cpp:66-76 for a restart).  v may be NULL (zero). */
int swc_sand_set_particles(swc_sand * s, const double * x, const double * v, int64_t n);
int swc_sand_get_particles(swc_sand * s, double * x, double * v, int64_t n);
/* Boundary particles with their normals (BoundaryParticles::addSurface,
 * Cores/Structures/SmoothedParticles.cpp:111-155).  Their velocity is zero, as the
 * reference's _boundary_velocity field, which nothing sets. */
int swc_sand_set_boundary(swc_sand * s, const double * x, const double * normals, int64_t nb);

/* DEMParticleSand::initialize (DEMParticleSand.cpp:78-88): boundary densities and
 * volumes from the boundary particles (kernel radius 4r), and the cell lattice
 * (cells of 2r over the box of all particles; particles that later leave it are
 * binned in its border cells). */
int swc_sand_initialize(swc_sand * s);
/* DEMParticleSand::advance (DEMParticleSand.cpp:90-94): move, contact and boundary
 * friction forces, gravity. */
int swc_sand_advance(swc_sand * s, double dt);
/* DEMParticleSand::getTimeStep (DEMParticleSand.h:38-40): step_rate * 2r / max|v|. */
int swc_sand_get_time_step(swc_sand * s, double step_rate, double * dt);
/* Boundary densities and volumes after initialize, in input order. */
int swc_sand_get_boundary_info(swc_sand * s, double * rho, double * vol, int64_t nb);
/* Mean device time of one kernel over `reps` launches on the current state:
 * 0 = contact pass (forces, boundary friction, gravity), 1 = binning (counting
 * sort into the cells, without the move). */
int swc_sand_time_kernel(swc_sand * s, int which, int reps, double * mean_ms);

#ifdef __cplusplus
}
#endif

#endif /* SWC_SAND_H */
