/*
 * dem_gb300.h — C ABI of libdem_sm100a.so, the GB300 (sm_103a) DEM time step.
 *
 * This boundary replaces the device-side half of the reference package DEMPort
 * (lucifer1004/taichi_dem_julia_port): the `GlobalData` device state
 * (src/executor.jl:1-29), `initialize!` (src/executor.jl:155-160), `simulate!`
 * (src/executor.jl:162-172) and the per-scene setup that `solve` performs before
 * its loop (src/executor.jl:217-340).  A host front end (the Python package
 * `taichi_dem_julia_port_gb300`, or a Julia `ccall` shim) keeps the reference's
 * TOML config, p4p/p4c files and step loop and calls these entry points.
 *
 * Conventions
 *  - Every function returns an int status: DEM_OK (0) or a DEM_ERR_* code.
 *  - The library owns all device memory; the caller owns every host buffer.
 *  - Host arrays of 3-vectors are interleaved (x0,y0,z0,x1,...), length 3*n.
 *    Quaternions are (w,x,y,z), length 4*n.
 *  - Particle indices are 0-based (reference index - 1).  Values that the
 *    reference computes as 1-based quantities (cell ijk, Morton code,
 *    hash-table bucket) are returned with the reference's own values.
 *  - One host thread per handle.  Each handle has its own CUDA stream; calls
 *    on one handle are ordered on that stream.
 */
#ifndef DEM_GB300_H
#define DEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DEM_OK 0
#define DEM_ERR_INVALID 1   /* bad argument or state                          */
#define DEM_ERR_CUDA 2      /* a CUDA runtime call failed                     */
#define DEM_ERR_CAPACITY 3  /* a contact / pair buffer would overflow         */
#define DEM_ERR_TIMEOUT 4   /* a bounded device-side wait gave up             */
#define DEM_ERR_NO_DEVICE 5 /* no usable sm_103 device                        */
#define DEM_ERR_RANGE 6     /* a particle left the 10-bit Morton cell range   */

/* ---- precision modes (dem_set_precision) ------------------------------- */
#define DEM_FP64 0       /* every force in FP64 (the reference's arithmetic)  */
#define DEM_FP32_FORCE 1 /* Hertz-Mindlin/EBPM force evaluation in FP32; state,
                            integration, shear history and the bond-breakage
                            test stay FP64                                     */

/* ---- contact flags ----------------------------------------------------- */
#define DEM_CONTACT_ACTIVE 1u /* reference BitTable `contact_active`          */
#define DEM_CONTACT_BONDED 2u /* reference BitTable `contact_bonded`          */

/*
 * The 32 numeric keys of `DEMConfig` (src/config.jl:3-43), same names and
 * meaning.  The 33rd key, `init_particles`, is a file name that the host front
 * end resolves and passes as DemParticlesIn.
 */
typedef struct DemConfigC {
    double domain_min[3];
    double domain_max[3];
    double particle_contact_radius_multiplier;
    double neighboring_search_safety_factor;
    double particle_elastic_modulus;
    double particle_poisson_ratio;
    double wall_normal[3];
    double wall_distance;
    double wall_density;
    double wall_elastic_modulus;
    double wall_poisson_ratio;
    double bond_radius_ratio;
    double bond_elastic_modulus;
    double bond_poisson_ratio;
    double bond_compressive_strength;
    double bond_tensile_strength;
    double bond_shear_strength;
    double pp_coefficient_friction;
    double pp_coefficient_restitution;
    double pp_coefficient_rolling_resistance; /* declared, unused (as in the reference) */
    double pw_coefficient_friction;
    double pw_coefficient_restitution;
    double pw_coefficient_rolling_resistance; /* declared, unused (as in the reference) */
    int64_t max_coordinate_number;     /* contacts per particle (the contact capacity is
                                        * n · this); also new partners and incoming
                                        * contacts per particle and step (at most 64)
                                        * and neighbour-list partners per particle
                                        * (at least 16, at most 256)                */
    int64_t collision_pair_init_capacity_factor;
    double tolerance;
    int64_t max_particle_count;
    double gravity[3];
    double global_damping;
    double dt;
    double target_time;
    double saving_interval_time;
} DemConfigC;

/* The p4p columns that `solve` reads per grain (src/executor.jl:219-243). */
typedef struct DemParticlesIn {
    int64_t n;
    const int32_t* id;     /* ID column                       */
    const int32_t* gid;    /* GROUP column                    */
    const double* volume;  /* VOLUME column (n)               */
    const double* mass;    /* MASS column (n)                 */
    const double* pos;     /* PX PY PZ (3n)                   */
    const double* vel;     /* VX VY VZ (3n)                   */
} DemParticlesIn;

/* Dynamic particle state (the mutable fields of `Grain`, src/types.jl:46-61,
 * plus the `forces`/`moments` arrays and the wall shear history of
 * `GlobalData`).  Any pointer may be NULL to skip that field. */
typedef struct DemParticleState {
    int64_t n;
    double* pos;        /* 3n  𝐤                                         */
    double* vel;        /* 3n  𝐯                                         */
    double* omega;      /* 3n  𝛚                                         */
    double* quat;       /* 4n  𝐪 (w,x,y,z)                               */
    double* force;      /* 3n  total force of the last step (get only)    */
    double* moment;     /* 3n  total moment of the last step (get only)   */
    double* wall_shear; /* 3n  𝐬 of wall_contacts[1, i]                  */
} DemParticleState;

/* Static per-particle data derived at setup (src/executor.jl:223-242). */
typedef struct DemParticleStatic {
    int64_t n;
    double* radius;   /* r = ∛(V / (4/3 π))      */
    double* radius0;  /* r₀ = r · multiplier     */
    double* mass;     /* m                       */
    double* inertia;  /* 2/5 m r² (diagonal of 𝐈) */
} DemParticleStatic;

/* Active contacts (the reference's `contacts[1:contact_ptr[1]]` filtered by
 * the `contact_active` bit, src/utils.jl:53-69).  Arrays hold `cap` entries. */
typedef struct DemContacts {
    int32_t* i;        /* owner particle, i < j      */
    int32_t* j;
    uint8_t* bonded;   /* 1 = EBPM bond, 0 = Hertz-Mindlin */
    double* point;     /* 3 per contact, 𝐤 (contact position)   */
    double* force;     /* 3 per contact, 𝐅ᵢ in the local frame  */
    double* torque_i;  /* 3 per contact, 𝛕ᵢ                     */
    double* torque_j;  /* 3 per contact, 𝛕ⱼ                     */
    double* shear;     /* 3 per contact, 𝐬                      */
} DemContacts;

/* ---- material, surface and wall tables ---------------------------------
 * The reference's GlobalData holds a table of materials, a square table of
 * surfaces indexed by the two materials in contact, a list of walls and one
 * material index per grain (src/types.jl:9-27, 58-62; src/executor.jl:1-29);
 * its kernels read them per contact (src/kernels.jl:175-177, 255-263) and
 * loop over the walls per particle (src/kernels.jl:317-426).  Its `solve`
 * fills them with one particle material, one wall material and one wall
 * (src/executor.jl:282-315), which is what dem_create does.  Indices here are
 * 0-based (the reference's mid - 1). */
#define DEM_MAX_MATERIALS 8
#define DEM_MAX_WALLS 8

typedef struct DemMaterial {   /* Material (src/types.jl:9-13) */
    double density;            /* ρ (not used by any force)            */
    double elastic_modulus;    /* E                                    */
    double poisson_ratio;      /* ν                                    */
} DemMaterial;

typedef struct DemSurface {    /* Surface (src/types.jl:17-27) */
    double friction;           /* μ                                    */
    double restitution;        /* e                                    */
    double rolling_resistance; /* μᵣ (declared, unused, as in the reference) */
    double bond_radius_ratio;  /* ρ: bond radius = ρ·min(rᵢ, rⱼ)       */
    double bond_elastic_modulus;
    double bond_poisson_ratio;
    double bond_compressive_strength;
    double bond_tensile_strength;
    double bond_shear_strength;
} DemSurface;

typedef struct DemWall {       /* Wall (src/types.jl:58-62) */
    double normal[3];          /* 𝐧                                    */
    double distance;           /* d: the plane 𝐧·𝐱 = d                 */
    int64_t material;          /* index into the materials            */
} DemWall;

typedef struct DemTables {
    int64_t n_materials;              /* 1 .. DEM_MAX_MATERIALS         */
    const DemMaterial* materials;     /* n_materials                    */
    const DemSurface* surfaces;       /* n_materials², [a * n_materials + b] = surfaces[a+1, b+1] */
    int64_t n_walls;                  /* 0 .. DEM_MAX_WALLS             */
    const DemWall* walls;             /* n_walls                        */
    const int32_t* grain_material;    /* one per grain (Grain.mid - 1)  */
} DemTables;

/* One line of a p4c record, as `save_single` writes it (src/utils.jl:48-69):
 * the contact's particles (0-based, i < j), whether it is a bond, its
 * position 𝐤 and its force 𝐅ᵢ in the local frame.  64 bytes. */
typedef struct DemIOContact {
    int32_t i, j;
    int32_t bonded;
    int32_t pad;
    double point[3];
    double force[3];
} DemIOContact;

/* Values `solve` derives before the loop (src/executor.jl:244-267). */
typedef struct DemDerived {
    double cell_size;        /* 4 rₘₐₓ                                  */
    double r_max;            /* rₘₐₓ                                    */
    int64_t hash_table_size; /* clamp(∏ ceil((max-min)/cell), 2^20, 2^22) */
    int64_t total_steps;     /* trunc(target_time / dt)                 */
    int64_t save_per_steps;  /* trunc(saving_interval_time / dt)        */
    double material_density; /* m/V of the last grain                   */
    int64_t contact_capacity;/* n · max_coordinate_number               */
} DemDerived;

typedef struct DemStats {
    int64_t n_particles;
    int64_t steps_done;
    int64_t contacts;        /* active contacts now (bonded + Hertz)    */
    int64_t bonded;          /* active bonds now                        */
    int64_t bonds_broken;    /* cumulative EBPM breakages               */
    int64_t contacts_ended;  /* cumulative Hertz contacts ended         */
    int64_t contacts_created;/* cumulative Hertz contacts created       */
    int64_t warn_gap;        /* "gap > 0" events (src/kernels.jl:243-245)  */
    int64_t warn_damping;    /* "γ < 0" events (src/kernels.jl:271-279)    */
    int32_t error;           /* sticky DEM_ERR_* raised on the device   */
    int32_t precision;       /* DEM_FP64 or DEM_FP32_FORCE              */
    int64_t full_searches;   /* steps that ran the full pair search (the
                                others tested the neighbour lists)      */
    int64_t exchanges_direct;/* dem_step_exchange calls whose last step's
                                integrator wrote the state into the
                                caller's buffers while it ran (the others
                                read it after the step)                 */
} DemStats;

typedef struct DemHandle DemHandle;

/* ---- lifetime ---------------------------------------------------------- */

/* Makes `device` current for the calling thread; handles created afterwards
 * live on it.  No counterpart in the reference (one GPU, CUDA.jl default). */
int dem_set_device(int device);

/* Builds the device state of one scene: the grain setup, derived sizes,
 * material/surface/wall tables and buffers of `solve`
 * (src/executor.jl:217-340).  Replaces `cu(grains_cpu)` + `GlobalData(...)`. */
int dem_create(const DemConfigC* cfg, const DemParticlesIn* particles,
               DemHandle** out);

/* Frees every device buffer of the handle (the reference relies on GC,
 * src/executor.jl:176-177). */
int dem_destroy(DemHandle* h);

/* ---- the step ---------------------------------------------------------- */

/* `initialize!` (src/executor.jl:155-160): broad phase + `init_bonds!`
 * (src/kernels.jl:60-85). */
/* dem_create with the scene's own material, surface and wall tables (the
 * reference's GlobalData.materials / surfaces / walls and Grain.mid, which
 * `initialize!` and `simulate!` read; src/executor.jl:155-172).  The config
 * supplies everything else as for dem_create: domain, derived sizes (cell
 * size from the largest radius and the config's bond strength and modulus,
 * src/executor.jl:244-267), dt, gravity, damping, tolerance, contact
 * capacity; its material, surface and wall keys are not used.  Returns
 * DEM_ERR_INVALID for a table outside the limits above or an index out of
 * range.  Such a handle computes in FP64: dem_set_precision(DEM_FP32_FORCE)
 * returns DEM_ERR_INVALID for it. */
int dem_create_tables(const DemConfigC* cfg, const DemParticlesIn* particles,
                      const DemTables* tables, DemHandle** out);

/* Shear history 𝐬 of wall `wall`'s contacts, wall_contacts[wall+1, :] of the
 * reference (3n doubles, zero where the grain does not touch the wall).
 * DemParticleState.wall_shear is wall 0's. */
int dem_get_wall_shear(DemHandle* h, int32_t wall, double* shear);
int dem_set_wall_shear(DemHandle* h, int32_t wall, const double* shear);

int dem_init_bonds(DemHandle* h);

/* `simulate!` × nsteps (src/executor.jl:162-172): clear_state!, contact!,
 * resolve_wall!, apply_body_force!, update!, late_clear_state!.  Asynchronous
 * on the handle's stream; errors raised on the device surface at the next
 * dem_sync / dem_get_* call. */
int dem_step(DemHandle* h, int64_t nsteps);

/* Same as dem_step, bracketed by CUDA events on the handle's stream; *ms is
 * the device time of the nsteps (synchronises). */
int dem_step_timed(DemHandle* h, int64_t nsteps, float* ms);

/* One step as the step graph runs it, with CUDA events before, between and
 * after its three kernels (one captured graph per contact-buffer parity, so
 * no host launch latency falls inside a phase).  phase_ms[0..2] (nphase >= 3; further
 * entries are set to 0) receive the device time of: the contact update (the
 * full pair search of the scenes whose neighbour lists went stale — hash,
 * bucket scan, scatter, canonical order, cp_list enumeration with
 * update_contacts! — and the neighbour-list update of the others, with the
 * next contact rows), contact forces, integration.
 * No counterpart in the reference: per-kernel timing for roofline reports. */
int dem_step_profiled(DemHandle* h, float* phase_ms, int nphase);

/* Waits for the handle's stream and reports the sticky device error. */
int dem_sync(DemHandle* h);

/* Selects the force arithmetic: DEM_FP64 (default, the reference's) or
 * DEM_FP32_FORCE.  No counterpart in the reference, which is FP64 only. */
int dem_set_precision(DemHandle* h, int mode);

/* Launch shape of the grid-stride kernels (contact forces, integration):
 * block sizes (multiples of 32, at most 256) and grid upper bounds.  Results
 * are the same for every shape; the shape only changes speed (the
 * autotuner's knob).  No counterpart in the reference. */
typedef struct DemLaunchShape {
    int32_t force_block;
    int32_t force_grid;
    int32_t compact_block;        /* kept for layout; no effect (rows are rebuilt
                                   * where contacts are decided)                    */
    int32_t compact_grid;         /* kept for layout; no effect                     */
    int32_t integrate_block;
    int32_t detect_blocks_per_sm; /* register budget of the pair search and the
                                   * neighbour-list update: 3 or 4 (0 = 4)          */
    int32_t force_blocks_per_sm;  /* FP32 force kernel: 0 (compiler's choice) or 4
                                   * (register budget for four 256-thread blocks per
                                   * SM); default 4 for a single scene, 0 for an arena */
    int32_t dependent_launch;     /* a step's kernels: 0 ordinary launches; 1
                                   * programmatic dependent launches (each may be
                                   * scheduled while its predecessor finishes); 2 the
                                   * same, successor scheduled once all blocks run  */
    int32_t list_lanes;           /* neighbour-list update: lanes per particle, 1 or 4
                                   * (0 = 1 when the particles outnumber half the
                                   * launch's threads, else 4)                        */
    int32_t integrate_lanes;      /* integrator: threads per particle, 1 or 4 (one
                                   * per force component and one for the walls and
                                   * the quaternion, in four warps per 32 particles);
                                   * 0 = 4 while the particles number at most 256 per
                                   * SM, else 1.  Results do not change.              */
} DemLaunchShape;

int dem_set_launch_shape(DemHandle* h, const DemLaunchShape* shape);

/* Neighbour-list skin of one scene (scene >= 0; 0 for a single-scene handle)
 * or of every scene (scene < 0), as a fraction in [0, 1] of the largest skin
 * the octant search allows (cell/2 - 2·max r).  Default 0.9.  A scene runs the
 * full pair search (the reference's cp_list) when one of its particles has
 * moved by skin/2 since its last full search, and otherwise tests only its
 * lists; contact sets are the same either way.  0 searches in full every
 * step.  No counterpart in the reference (it searches every step). */
int dem_set_skin_factor(DemHandle* h, int32_t scene, double skin_factor);
int dem_get_launch_shape(DemHandle* h, DemLaunchShape* out);

/* ---- state exchange ---------------------------------------------------- */

/* Reads `grains` (positions, velocities, ...) back to the host, as
 * `Array(grains)` does in save_single (src/utils.jl:40).  Buffers in
 * page-locked host memory (cudaHostAlloc, cudaHostRegister) or in device
 * memory are written in place by one kernel; pageable buffers take one extra
 * copy through a device staging buffer.  Returns when the data is in place. */
int dem_get_particles(DemHandle* h, DemParticleState* out);

/* Overwrites the dynamic particle state from host buffers (fields left NULL
 * are kept; buffers as for dem_get_particles).  Used to start the device from
 * a given state.  The buffers are no longer read once the call returns.  New
 * positions keep the neighbour lists while every particle stays within half
 * the skin of where they were built; otherwise the next step searches in full. */
int dem_set_particles(DemHandle* h, const DemParticleState* in);

/* dem_set_particles ordered on the handle's stream without waiting for it:
 * page-locked or device buffers are read by a kernel later in the stream and
 * must stay unchanged until the next synchronising call (dem_sync,
 * dem_get_*, dem_step_timed); pageable buffers are free on return.  For a
 * host loop that writes the state, steps and reads it back every step. */
int dem_set_particles_async(DemHandle* h, const DemParticleState* in);

/* One call of a host loop that exchanges the state every step:
 * dem_set_particles_async(in) (skipped for NULL), dem_step(nsteps), then
 * dem_get_particles(out) (skipped for NULL; returns when `out` holds the
 * state).  Single-scene handles.  With `in` and `out` in page-locked host (or
 * device) memory and the integrator split over four warps per 32 particles
 * (scenes of up to 256 particles per SM), the host-link traffic overlaps the
 * step: the positions are uploaded first, the other fields beside the
 * contact update (a one-step call replays one captured graph per set of
 * buffers; in a call of several steps the velocities and spins go with the
 * positions and the first step's integrator reads the orientations and the
 * first wall's shear history from `in`), and the last step's integrator
 * writes the state into `out` block by block as it finishes
 * (DemStats.exchanges_direct counts these calls).  `in` and `out` may be the
 * same buffers; a one-step exchange in place then leaves out the values the
 * step did not change (bit for bit), which the buffers hold already.
 * Replaces `simulate!` (src/executor.jl:162-172) with the host copy of the
 * grains around it (`Array(grains)`, src/utils.jl:40) done every step. */
int dem_step_exchange(DemHandle* h, const DemParticleState* in, int64_t nsteps,
                      DemParticleState* out);

/* Page-locked host memory for state buffers (cudaMallocHost / cudaFreeHost),
 * for callers without a CUDA runtime of their own.  The library remembers
 * these ranges, so exchanges with them skip the per-buffer pointer query.
 * No counterpart in the reference (CUDA.jl owns its host copies). */
int dem_host_alloc(int64_t bytes, void** out);
int dem_host_free(void* p);

int dem_get_static(DemHandle* h, DemParticleStatic* out);

int dem_get_derived(DemHandle* h, DemDerived* out);

/* The active contacts as p4c records, sorted by (i, j): what `save_single`
 * writes (src/utils.jl:48-69, which copies every contact and both BitTables
 * to the host and filters there).  The active contacts are compacted on the
 * device into DemIOContact records, and only those cross to the host.
 * *n_out receives the count even when it exceeds cap (then DEM_ERR_CAPACITY
 * is returned and nothing is written). */
int dem_get_io_contacts(DemHandle* h, DemIOContact* out, int64_t cap, int64_t* n_out);
int dem_scene_get_io_contacts(DemHandle* h, int32_t scene, DemIOContact* out, int64_t cap,
                              int64_t* n_out);

/* Active contacts, sorted by (i, j).  *n_out receives the count even when it
 * exceeds cap (then DEM_ERR_CAPACITY is returned and nothing is written). */
int dem_get_contacts(DemHandle* h, DemContacts* out, int64_t cap,
                     int64_t* n_out);

/* Replaces the contact list (active contacts only; sets the active bit, and
 * the bonded bit where bonded[k] != 0).  Pairs must satisfy i < j and be
 * unique. */
int dem_set_contacts(DemHandle* h, const DemContacts* in, int64_t n);

int dem_get_stats(DemHandle* h, DemStats* out);

/* ---- arenas: many independent scenes stepped together ------------------- */
/*
 * No counterpart in the reference, which steps one scene per process.  An
 * arena is a handle whose particle slots, contact buffers and bucket table are
 * shared by independent scenes; every dem_step advances all scenes in Step
 * mode by one `simulate!` each, in the same kernels.  Scenes can be added and
 * removed between steps (the device step graph never changes), which is what
 * the batched and served modes build on.  Each scene's results are the same,
 * bit for bit, as when it is stepped alone in its own arena.
 */
typedef struct DemArenaConfig {
    int64_t max_particles;   /* particle slots shared by all scenes          */
    int64_t max_contacts;    /* contact capacity shared by all scenes        */
    int64_t max_buckets;     /* bucket-table entries shared by all scenes    */
    int32_t max_scenes;
    int32_t max_coordinate_number; /* new partners / incoming contacts per
                                      particle and step (at most 64) and
                                      neighbour-list partners per particle
                                      (at least 16, at most 256)             */
    int32_t precision;       /* DEM_FP64 or DEM_FP32_FORCE                   */
    int32_t pad;
    double cell_factor;      /* search cell = cell_factor · 4 rₘₐₓ; 0 = 1.  Values
                                down to the minimum that still finds every
                                touching pair (cell >= 4·max r) are accepted. */
} DemArenaConfig;

#define DEM_SCENE_FREE 0
#define DEM_SCENE_FROZEN 1 /* state kept, not stepped (e.g. step target reached) */
#define DEM_SCENE_STEP 2
#define DEM_SCENE_INIT 3   /* bonds are created on the next dem_step         */

typedef struct DemSceneInfo {
    int32_t mode;            /* DEM_SCENE_*                                   */
    int32_t pad;
    int64_t n;               /* particles                                     */
    int64_t first_slot;      /* particle slot of the scene's particle 0      */
    int64_t steps_done;
    int64_t steps_target;    /* the scene freezes when steps_done reaches it (0 = never) */
    int64_t buckets;         /* bucket-table entries of the scene            */
} DemSceneInfo;

int dem_arena_create(const DemArenaConfig* cfg, DemHandle** out);

/* Adds a scene (the set-up of `solve`, src/executor.jl:217-315) to free slots.
 * init_bonds != 0 runs `initialize!` (src/kernels.jl:60-85) on the next
 * dem_step before the scene starts stepping; steps_target > 0 freezes the
 * scene after that many steps.  Returns DEM_ERR_CAPACITY when the arena has no
 * room (particles, buckets or scene records). */
int dem_arena_add(DemHandle* h, const DemConfigC* cfg, const DemParticlesIn* particles,
                  int init_bonds, int64_t steps_target, int32_t* scene);

/* Releases a scene's slots and contacts. */
int dem_arena_remove(DemHandle* h, int32_t scene);

/* Search-cell factor of one scene (scene >= 0) or of every scene (scene < 0),
 * as DemArenaConfig.cell_factor.  Takes effect at the next step and leaves
 * every result unchanged (contact ends still follow the reference's cells);
 * only the pair-search work changes (the autotuner's knob). */
int dem_arena_set_cell_factor(DemHandle* h, int32_t scene, double cell_factor);

int dem_arena_scene_info(DemHandle* h, int32_t scene, DemSceneInfo* out);

/* Per-scene state exchange; indices are scene-local (0-based). */
int dem_scene_get_particles(DemHandle* h, int32_t scene, DemParticleState* out);
int dem_scene_get_contacts(DemHandle* h, int32_t scene, DemContacts* out, int64_t cap,
                           int64_t* n_out);
int dem_scene_get_stats(DemHandle* h, int32_t scene, DemStats* out);
int dem_scene_get_derived(DemHandle* h, int32_t scene, DemDerived* out);

/* ---- parity / inspection ----------------------------------------------- */

/* Runs only the reference broad phase on the current positions and returns
 * its intermediate arrays (src/executor.jl:38-78):
 *   cell[3n]        kid        = cell(𝐤)                (src/utils.jl:1)
 *   morton[n]       cartesian3morton(kid)               (src/utils.jl:2)
 *   bucket[n]       hid        = hashcode(kid)  1-based (src/utils.jl:2)
 *   bucket_count[H] hash_table after count_particles!   (src/kernels.jl:7-13)
 *   sorted[n]       pid, within-bucket ascending        (src/kernels.jl:15-22)
 *   cp[2*cp_cap]    cp_list pairs (i,j), i<j            (src/kernels.jl:24-58)
 * Any output pointer may be NULL.  *cp_n receives the pair count; if it
 * exceeds cp_cap no pair is written and DEM_ERR_CAPACITY is returned. */
int dem_debug_broadphase(DemHandle* h, int32_t* cell, uint32_t* morton,
                         uint32_t* bucket, uint32_t* bucket_count,
                         uint32_t* sorted, int32_t* cp, int64_t cp_cap,
                         int64_t* cp_n);

/* Steps the scene once with the full pair search forced and returns what
 * the step's own fused enumeration visited: *pairs = the candidate pairs
 * (i, j > i) taken from the distinct buckets among i's 8 octant buckets,
 * *checksum = the wrapping 64-bit sum of a mix of each pair, with
 *   mix(i, j): z = i·2^32 + j; z ^= z >> 33; z *= 0xff51afd7ed558ccd;
 *              z ^= z >> 33; z *= 0xc4ceb9fe1a85ec53; z ^= z >> 33.
 * They equal the count and checksum of the distinct pairs of the
 * reference's cp_list (src/kernels.jl:24-58, dem_debug_broadphase) when the
 * step visits exactly those pairs.  Single-scene handles only; the step
 * otherwise runs as dem_step does. */
int dem_debug_step_enumeration(DemHandle* h, int64_t* pairs, uint64_t* checksum);

/* Bucket sort of the reference broad phase (cell, hashcode, counting sort:
 * src/utils.jl:1-2, src/kernels.jl:7-22) that allocates nothing.  No
 * counterpart in the reference.
 *
 * For callers that cannot allocate device memory: a host that reserves all
 * of its GPU buffers up front and forbids allocation afterwards, a process
 * whose device allocator belongs to another framework, or code running while
 * allocation is blocked.  The caller passes device pointers: positions
 * px/py/pz (n each), and the outputs bucket[n] (the reference's 1-based
 * hashcode) and sorted[n] (particle indices grouped by bucket, ascending
 * inside a bucket; the same as dem_debug_broadphase's `sorted`).
 * domain_min is a HOST pointer to 3 doubles (read during the call).  Work is
 * queued on `stream` (a cudaStream_t, NULL for the default stream); results
 * are ready when that stream is synchronised.
 *
 * The sort is a stable radix sort of the indices by bucket (one pass for
 * hash_table_size <= 1,024, two above): its work is O(n + H) whatever the
 * number of particles per bucket.
 *
 * The temporary memory is one 12.6 MB array inside the library, reserved on
 * every GPU that loads it until the process exits, so n and hash_table_size
 * are each limited to 1,048,576 (larger values return DEM_ERR_CAPACITY
 * before any work is queued).  The first call on a device looks up that
 * array's device address; make that first call before any stream capture on
 * the device.  Every call reuses the same array: calls whose work overlaps on
 * the GPU (different streams or threads) race and must be serialised by the
 * caller.  DEM_ERR_CUDA is returned, with nothing queued, when a CUDA error
 * is already pending on the calling thread (it is left in place for its
 * owner), and when one of this call's launches fails (the call stops at the
 * first failure). */
int dem_bucket_sort_noalloc(const double* px, const double* py, const double* pz,
                            int64_t n, const double* domain_min, double cell_size,
                            int64_t hash_table_size, uint32_t* bucket,
                            uint32_t* sorted, void* stream);

/* ---- misc -------------------------------------------------------------- */

/* Text for a status code.  For DEM_ERR_INVALID from dem_create,
 * dem_arena_add or dem_set_particles it names the offending grain and field
 * when an input value was the cause (the last such check on the calling
 * thread); for DEM_ERR_CUDA it is the CUDA runtime's message. */
const char* dem_strerror(int code);

/* Self-test: compares the library's integer-pipe FP64->FP32 and FP32->FP64
 * conversions (used by the FP32 force mode and the neighbour lists) with the
 * hardware conversions, its Newton-Raphson FP64 reciprocal with the
 * correctly rounded one, its integer-pipe halving with x * 0.5 and the
 * identities behind the integrator's zero-spin, zero-torque and
 * identity-orientation skips, on n seeded random values; mismatches[0] ..
 * [3] (four entries) receive the narrowing / widening mismatch counts, the
 * reciprocals more than 2 ulp off and the halvings or identities that fail
 * (all 0 when correct).  No counterpart in the reference. */
int dem_selftest_conversions(int64_t n, uint64_t seed, int64_t* mismatches);

/* Self-test of the device's bounded waits (the failure detection of the
 * fused pair search): which = 0 runs a grid barrier of two blocks, 1 a scan
 * look-back over two tiles, each with a wait limit of `spin_limit` polls
 * (1 .. 2^20).  With `missing` = 1 one party never arrives (its block returns
 * before the barrier / its tile never publishes), so the wait gives up and
 * *status receives DEM_ERR_TIMEOUT; with `missing` = 0 everyone arrives and
 * *status is DEM_OK.  Nothing hangs: every wait of the library is bounded in
 * the same way (about a second at the default limit) and reports
 * DEM_ERR_TIMEOUT through the handle's error word.  No counterpart in the
 * reference (its kernels do not wait on one another). */
int dem_selftest_wait_timeout(int which, int missing, int64_t spin_limit, int* status);

/* Library version string, e.g. "dem_gb300 0.1.0 sm_103a". */
const char* dem_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DEM_GB300_H */
