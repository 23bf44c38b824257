/*
 * fluidsph.h — C ABI of the GB300 (sm_103a) SPH step library, libfluidsph.so.
 *
 * This is the drop-in boundary for fluid-toy's per-substep SPH compute path,
 * `SphSimulation3DGrid` (src/simulation/sph_3d_grid.rs:33-1569 in the
 * reference). Every parameter struct below is byte-for-byte the reference's
 * `#[repr(C)]` POD struct, so a Rust caller passes its existing values through
 * `extern "C"` unchanged.
 *
 * Conventions
 *   - Every function returns an `int` status: FS_OK (0) or a negative FS_E_*.
 *     Nothing aborts and no C++ exception crosses the ABI. `fs_last_error()`
 *     returns a thread-local message describing the last failure.
 *   - A simulation owns one CUDA stream. `fs_step` is asynchronous on it (the
 *     reference's `queue.submit` is asynchronous too); the download and
 *     `fs_read_rigid_body_accum` calls synchronise the stream.
 *   - Device memory is allocated in `fs_create` for `max_particles` and never
 *     grows, like the reference's buffers (sph_3d_grid.rs:196-305).
 *   - Kernels that wait on other blocks (the single-pass scan) give up after a
 *     bounded number of polls and raise a device error word; the next
 *     synchronising call returns FS_E_DEVICE_TIMEOUT instead of hanging.
 */
#ifndef FLUIDSPH_H
#define FLUIDSPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ABI version: bumped whenever a struct layout or signature changes. It also
 * encodes the struct sizes so a caller built against another layout fails in
 * fs_create instead of corrupting memory. */
#define FS_ABI_VERSION 0x00010057u

/* ---- status codes -------------------------------------------------------- */
#define FS_OK 0
#define FS_E_INVALID_ARGUMENT (-1) /* null pointer, zero/NaN size, bad enum  */
#define FS_E_ABI_MISMATCH (-2)     /* caller built against another layout   */
#define FS_E_CAPACITY (-3)         /* N or a size beyond the allocated max   */
#define FS_E_CUDA (-4)             /* a CUDA runtime call failed             */
#define FS_E_DEVICE_TIMEOUT (-5)   /* a bounded device-side wait gave up     */
#define FS_E_NO_DEVICE (-6)        /* no CUDA device / library not usable    */
#define FS_E_STATE (-7)            /* call not valid in the current state    */

/* ---- boundary structs (reference layouts) -------------------------------- */

/* SphParticle3D, src/simulation/particle.rs:8-17 — 64-byte AoS record. */
typedef struct SphParticle3D {
    float position[3]; /* @0  */
    float _pad0;       /* @12 */
    float velocity[3]; /* @16 */
    float _pad1;       /* @28 */
    float force[3];    /* @32: non-pressure accel, then dv after finalize */
    float density;     /* @44 */
    float near_density;/* @48 */
    float normal[3];   /* @52: Akinci surface normal */
} SphParticle3D;

/* GpuSphParams3D, src/state/simulation.rs:344-361 — 64 bytes. `stiffness` is
 * carried for layout parity; no step stage reads it (the reference's pressure
 * stiffness is `pcisph_delta`). */
typedef struct GpuSphParams3D {
    float kernel_radius;
    float kernel_radius_sq;
    float kernel_radius_pow5;
    float kernel_radius_pow6;
    float kernel_radius_pow9;
    float mass;
    float rest_density;
    float stiffness;
    float near_stiffness;
    float viscosity;
    float dt;
    uint32_t num_particles;
    float surface_tension;
    float pcisph_delta;
    float xsph_epsilon;
    float _padding_st;
} GpuSphParams3D;

/* GpuContainerGeometry, src/state/simulation.rs:367-386 — 128 bytes. Forward
 * rows are R = Rz*Rx (local->world), inverse rows are R^T. */
typedef struct GpuContainerGeometry {
    float half_width;
    float half_height;
    float half_depth;
    float center_y;
    float forward_row0[4];
    float forward_row1[4];
    float forward_row2[4];
    float inverse_row0[4];
    float inverse_row1[4];
    float inverse_row2[4];
    float wall_stiffness;
    float damping;
    uint32_t clip_enabled;
    float clip_margin;
} GpuContainerGeometry;

/* GpuGravity, src/state/simulation.rs:391-394 — 16 bytes. */
typedef struct GpuGravity {
    float direction[3];
    float _padding;
} GpuGravity;

/* GpuMouseForce, src/state/interaction.rs:102-111 — 48 bytes.
 * mode: 0 push, 1 pull, 2 vortex, 3 explode, 4 drain (interaction.rs:5-11). */
typedef struct GpuMouseForce {
    float position[3];
    float radius;
    float strength;
    uint32_t is_active;
    uint32_t mode;
    float _pad;
    float direction[3];
    float _pad2;
} GpuMouseForce;

/* GpuRigidBody, src/state/rigid_body.rs:212-224 — 96 bytes.
 * shape: 0 cube, 1 sphere, 2 cylinder, 3 torus, 4 custom SDF. Rotation rows
 * are world->local (rigid_body.rs:188-205). */
typedef struct GpuRigidBody {
    float position[3];
    float half_extent;
    float velocity[3];
    uint32_t is_active;
    float stiffness;
    uint32_t shape;
    float _pad1;
    float _pad2;
    float rot_row0[4];
    float rot_row1[4];
    float rot_row2[4];
} GpuRigidBody;

/* GpuRigidBodyAccum, src/state/rigid_body.rs:247-256 — 32 bytes, fixed point
 * x1000 (each particle's contribution truncated toward zero). */
typedef struct GpuRigidBodyAccum {
    int32_t force_x;
    int32_t force_y;
    int32_t force_z;
    uint32_t contact_count;
    int32_t torque_x;
    int32_t torque_y;
    int32_t torque_z;
    uint32_t _pad;
} GpuRigidBodyAccum;

/* The simulated rigid body of RigidBodyConfig (src/state/rigid_body.rs:86-113)
 * in the form integrate_rigid_body reads and writes, plus the wall
 * stiffness its GpuRigidBody carries — 80 bytes. shape: 0 cube, 1 sphere,
 * 2 cylinder, 3 torus, 4 custom. */
typedef struct FsRigidBodyState {
    float position[3];
    float half_extent;
    float velocity[3];
    float density;            /* body density (mass = density * shape volume) */
    float orientation[4];     /* quaternion x, y, z, w */
    float angular_velocity[3];
    uint32_t shape;
    uint32_t enabled;
    uint32_t held;            /* user-positioned: clamped, not integrated */
    float wall_stiffness;     /* GpuRigidBody.stiffness */
    uint32_t _pad;
} FsRigidBodyState;

/* GpuGridParams, src/simulation/sph_3d_grid.rs:15-30 — 48 bytes. */
typedef struct GpuGridParams {
    uint32_t grid_size_x;
    uint32_t grid_size_y;
    uint32_t grid_size_z;
    uint32_t total_cells;
    float cell_size;
    float inv_cell_size;
    float grid_origin_x;
    float grid_origin_y;
    float grid_origin_z;
    uint32_t num_particles;
    uint32_t _padding[2];
} GpuGridParams;

/* GpuGridParams of the marching-cubes renderer, src/render/marching_cubes.rs:
 * 56-66 — 48 bytes. Named GpuMcGridParams here because the SPH grid struct
 * above carries the same name in the reference. */
typedef struct GpuMcGridParams {
    float grid_min[3];
    uint32_t grid_size;      /* voxels per dimension */
    float grid_max[3];
    float cell_size;         /* voxel edge length */
    float kernel_radius;     /* splat radius (sim h * mc_density_radius_scale) */
    float iso_value;
    uint32_t num_particles;
    uint32_t max_vertices;
} GpuMcGridParams;

/* GpuSprayParams, src/state/interaction.rs:129-153 — 80 bytes. */
typedef struct GpuSprayParams {
    float min_speed;
    float emission_rate;
    float lifetime;
    float lifetime_variation;
    float drag;
    float speed_multiplier;
    float velocity_jitter;
    float dt;                 /* frame time: substep dt x substeps */
    uint32_t max_particles;
    uint32_t num_sph_particles;
    uint32_t frame_count;
    float gravity_y;
    float k_trapped_air;
    float k_wave_crest;
    float ta_limit;           /* potential ceilings: see fs_spray_step */
    float bubble_buoyancy;
    float bubble_drag;
    float wc_limit;
    float _pad[2];
} GpuSprayParams;

/* GpuSprayParticle, src/state/interaction.rs:155-174 — 48 bytes. kind: 0
 * spray, 1 foam, 2 bubble; lifetime <= 0 is a dead slot. */
typedef struct GpuSprayParticle {
    float pos[3];
    float lifetime;
    float vel[3];
    float max_lifetime;
    uint32_t kind;
    float age;
    float _pad[2];
} GpuSprayParticle;

/* Device pointers of a simulation, the analogue of the reference's buffer
 * getters (sph_3d_grid.rs:1500-1530). The library keeps particles as
 * structure-of-arrays float4 records (one coalesced 16-byte load per field),
 * not the reference's 64-byte AoS; fs_download_particles/_sorted rebuild the
 * AoS view. */
typedef struct FsDevicePointers {
    void *pos;            /* float4[max] canonical (x,y,z,_pad0)            */
    void *vel;            /* float4[max] canonical (vx,vy,vz,_pad1)         */
    void *force;          /* float4[max] canonical (fx,fy,fz,0)             */
    void *sorted_pos;     /* float4[max] grid-sorted positions              */
    void *sorted_vel;     /* float4[max] grid-sorted pre-XSPH velocities    */
    void *sorted_density; /* float2[max] (density, near_density)            */
    void *sorted_normal;  /* float4[max] (nx,ny,nz,0)                       */
    void *cell_counts;    /* uint32[total_cells]                            */
    void *cell_starts;    /* uint32[total_cells] inclusive ends (reference) */
    void *cell_begin;     /* uint32[total_cells+1] exclusive begins         */
    void *particle_cell_indices; /* uint32[max] orig -> sorted slot         */
    void *sorted_to_orig; /* uint32[max] sorted slot -> orig                */
    void *stream;         /* cudaStream_t the simulation launches on        */
} FsDevicePointers;

typedef struct FsSim FsSim; /* opaque SphSimulation3DGrid */

/* ---- library ------------------------------------------------------------- */

/* Thread-local description of the last error (never NULL). */
const char *fs_last_error(void);
/* FS_ABI_VERSION of the built library. */
uint32_t fs_abi_version(void);

/* ---- host-side constants (restating src/state/simulation.rs) ------------- */

/* compute_rest_density, src/state/simulation.rs:402-425. */
float fs_compute_rest_density(float h, float mass);
/* compute_pcisph_delta, src/state/simulation.rs:429-480. */
float fs_compute_pcisph_delta(float h, float mass, float rest_density, float dt);
/* SphConfig::to_gpu_params_3d, src/state/simulation.rs:315-337, with the rest
 * density passed in (the reference derives it from h and mass; pass
 * fs_compute_rest_density(h, mass) for the reference's own value). */
int fs_sph_params_3d(float kernel_radius, float mass, float rest_density,
                     float stiffness, float near_stiffness, float viscosity,
                     float surface_tension, float xsph_epsilon, float dt,
                     uint32_t num_particles, GpuSphParams3D *out);
/* ContainerConfig::to_gpu_geometry, src/state/simulation.rs:139-184. */
int fs_container_geometry(float width, float depth, float floor_y, float height,
                          float tilt_x, float tilt_z, float wall_stiffness,
                          float damping, uint32_t clip_enabled, float clip_margin,
                          GpuContainerGeometry *out);
/* quat_to_rotation_rows, src/state/rigid_body.rs:188-205 (q = x,y,z,w). */
int fs_quat_to_rotation_rows(const float q[4], float rows[12]);
/* RigidBodyConfig::to_gpu_rigid_body, src/state/rigid_body.rs:131-146. */
int fs_rigid_body_to_gpu(const FsRigidBodyState *state, GpuRigidBody *out);
/* integrate_rigid_body, src/state/rigid_body.rs:277-365 (reaction forces and
 * torques of the accumulator -> velocities -> pose, then the container clamp
 * with bounce): the reference's per-frame CPU step, on the host. */
int fs_integrate_rigid_body(FsRigidBodyState *state, const GpuContainerGeometry *container,
                            float substep_dt, uint32_t num_substeps, const float gravity[3],
                            const GpuRigidBodyAccum *accum);
/* clamp_rigid_body_to_container, src/state/rigid_body.rs:415-479. */
int fs_clamp_rigid_body(FsRigidBodyState *state, const GpuContainerGeometry *container,
                        int bounce_velocity);
/* Grid sizing of SphSimulation3DGrid::new, sph_3d_grid.rs:121-143. */
int fs_grid_params_for(float kernel_radius, uint32_t num_particles,
                       GpuGridParams *out);

/* MarchingCubesRenderer::update_params, src/render/marching_cubes.rs:
 * 2099-2113: cell_size = largest extent of [grid_min, grid_max] / grid_size,
 * max_vertices = 4,000,000 (marching_cubes.rs:20). */
int fs_mc_grid_params(const float grid_min[3], const float grid_max[3], uint32_t grid_size,
                      float kernel_radius, float iso_value, uint32_t num_particles,
                      GpuMcGridParams *out);

/* ---- SphSimulation3DGrid ------------------------------------------------- */

/* SphSimulation3DGrid::new, sph_3d_grid.rs:104-1258. `sdf` may be NULL (the
 * reference then binds a 1x1x1 texture holding 1.0, i.e. "outside"); else it
 * is sdf_res^3 floats, x fastest, sampled with clamp-to-edge trilinear
 * filtering. `device` selects the CUDA device. max_particles is raised to n
 * like the reference (sph_3d_grid.rs:114). Gravity starts at (0,-9.8,0), the
 * mouse force and rigid body start inactive at their reference defaults. */
int fs_create(const SphParticle3D *particles, uint32_t num_particles,
              const GpuSphParams3D *params, const GpuContainerGeometry *geom,
              uint32_t max_particles, const float *sdf, uint32_t sdf_res,
              int device, uint32_t abi_version, FsSim **out);
int fs_destroy(FsSim *sim);

/* step(), sph_3d_grid.rs:1261-1444, run `nsteps` times back to back on the
 * simulation's stream. With nsteps > 1 the steps run from captured CUDA
 * graphs: one graph of up to 256 whole steps, replayed, plus one-step
 * replays for a remainder. A graph is captured on first use for its step
 * count and the current particle counts and iteration count (a few are
 * kept). Asynchronous. */
int fs_step(FsSim *sim, uint32_t nsteps);
/* No counterpart in the reference. Capture now the graphs a later
 * fs_step(sim, nsteps) uses, so that call only launches. */
int fs_prepare_steps(FsSim *sim, uint32_t nsteps);
/* No counterpart in the reference. The neighbour passes (density, XSPH,
 * PCISPH solve) each exist in several forms that differ only in how many
 * candidate records a lane loads ahead (the load depth: 0 = the plain loop,
 * 4, 8 or 16 for density and solve; 1, 4, 8 or 16 for XSPH; 32 = the staged
 * form of XSPH, in which a warp whose lanes share one cell moves chunks of 32
 * records through shared memory, each lane loading one record of the next
 * chunk). Every form gives
 * the same bits; which is fastest depends on the workload (deeper batches hide
 * more latency per lane but fit fewer warps on an SM), so a project-written
 * autotuner chooses per particle-count bucket: the bucket is
 * (floor(log2 hashed particles), one scene or many, PCISPH iterations). A
 * simulation whose bucket is already in the process-wide table takes its
 * depths at once; otherwise, once it has run 8 steps, its next 10 steps run
 * each depth twice (0, 1, 2, 3, 4, 4, 3, 2, 1, 0) with events around the three
 * passes, whatever the fs_step call sizes, and the next fs_step /
 * fs_prepare_steps / fs_frames call BLOCKS THE HOST ONCE until those 10 steps
 * have run on the GPU; each pass then keeps its fastest depth, which also
 * enters the table. Callers that must never block call fs_set_kernel_forms
 * first. fs_load_batching: batched = 1 when the density or solve pass runs
 * with batched loads, decided = 1 once the depths are fixed. */
int fs_load_batching(FsSim *sim, int *batched, int *decided);
typedef struct FsKernelForms {
    uint32_t density_loads, solve_loads, xsph_loads; /* load depths in use        */
    uint32_t decided;  /* 0 pending, 1 measured by this simulation, 2 from the
                          table (an earlier simulation of the bucket), 3 set by
                          fs_set_kernel_forms                                   */
    uint32_t bucket;   /* floor(log2 hashed particles)                          */
    float ms[3][5];    /* measured ms (density, XSPH, solve) per depth index
                          (depths 0/1, 4, 8, 16, 32), 0 unless measured by this
                          simulation                                            */
} FsKernelForms;
/* The simulation's forms (waits for a pending measurement, like fs_step). */
int fs_kernel_forms(FsSim *sim, FsKernelForms *out);
/* Fix the forms (no measurement, no host wait), or all -1 to tune again.
 * Depths outside the lists above return FS_E_INVALID_ARGUMENT. */
int fs_set_kernel_forms(FsSim *sim, int density_loads, int solve_loads, int xsph_loads);
typedef struct FsKernelFormsEntry {
    uint32_t device, bucket, many_scenes, iterations;
    uint32_t density_loads, solve_loads, xsph_loads, _pad;
    float ms[3][5];    /* the measured ms the depths were chosen by             */
} FsKernelFormsEntry;
/* The process-wide table: *count = entries; up to `capacity` copied to out
 * (out may be NULL to query the count). */
int fs_kernel_forms_table(FsKernelFormsEntry *out, uint32_t capacity, uint32_t *count);

/* update_* uploads, sph_3d_grid.rs:1446-1473. Ordered before later steps. */
int fs_update_sph_params(FsSim *sim, const GpuSphParams3D *params);
int fs_update_container_geometry(FsSim *sim, const GpuContainerGeometry *geom);
int fs_update_mouse_force(FsSim *sim, const GpuMouseForce *mouse);
int fs_update_gravity(FsSim *sim, const GpuGravity *gravity);
int fs_update_rigid_body(FsSim *sim, const GpuRigidBody *body);
/* set_pcisph_iterations, sph_3d_grid.rs:1475-1477 (clamped to >= 1). */
int fs_set_pcisph_iterations(FsSim *sim, uint32_t iterations);

/* clear_rigid_body_accum / read_rigid_body_accum, sph_3d_grid.rs:1479-1498.
 * The read synchronises the stream. */
int fs_clear_rigid_body_accum(FsSim *sim);
int fs_read_rigid_body_accum(FsSim *sim, GpuRigidBodyAccum *out);

/* num_particles(), sph_3d_grid.rs:1528-1530. */
int fs_num_particles(const FsSim *sim, uint32_t *out);
/* grid parameters the simulation was built with (grid_params_buffer). */
int fs_grid_params(const FsSim *sim, GpuGridParams *out);

/* spawn_particles, sph_3d_grid.rs:1534-1569: golden-angle spiral, clipped at
 * capacity; *spawned receives the count actually added. */
int fs_spawn_particles(FsSim *sim, const float position[3], uint32_t count,
                       float spread, uint32_t *spawned);
/* The particle records spawn_particles (sph_3d_grid.rs:1543-1557) builds
 * before writing them, on the host, for a simulation that holds
 * num_particles of max_particles: *spawned = min(count, max - num) records
 * on a golden-angle spiral around `position` (radius spread * sqrt(i / n),
 * layers of 20 stacked 0.3 spread apart), zero but the position
 * (SphParticle3D::new, particle.rs:19-31). out holds *spawned records.
 * fs_spawn_particles writes exactly these. No GPU. */
int fs_spawn_positions(const float position[3], uint32_t count, float spread,
                       uint32_t num_particles, uint32_t max_particles, SphParticle3D *out,
                       uint32_t *spawned);

/* ---- device-resident rigid-body coupling ----------------------------------- */

/* The reference's frame (src/app.rs:1205-1290): clear the accumulator, run the
 * substeps, read the accumulator back (a blocking map) and integrate the body
 * on the CPU (integrate_rigid_body), then upload its GpuRigidBody for the
 * next frame. Here the body's state lives on the device and the integration
 * runs as a kernel after the substeps, with the same arithmetic as
 * fs_integrate_rigid_body, so frames queue without host synchronisation.
 * fs_rigid_coupling_set_state couples a scene's body (NULL uncouples; the
 * scene's GpuRigidBody is then whatever was last written). While coupled,
 * the state drives the scene's GpuRigidBody (fs_update_rigid_body is
 * overridden at the next frame). */
int fs_rigid_coupling_set_state(FsSim *sim, uint32_t scene, const FsRigidBodyState *state);
/* The coupled body's current state (synchronises). */
int fs_rigid_coupling_get_state(FsSim *sim, uint32_t scene, FsRigidBodyState *out);
/* `frames` frames of `substeps` steps each, graph-replayed. Per frame:
 * clear every scene's accumulator, step, then integrate each coupled body
 * (enabled and not held) or clamp it to its container (held). The
 * accumulators of the last frame stay readable. */
int fs_frames(FsSim *sim, uint32_t substeps, uint32_t frames);

/* ---- whitewater (spray, foam, bubbles) ------------------------------------- */

/* SpraySystem, src/simulation/spray.rs (Ihmsen et al. 2012 diffuse particles):
 * emission from trapped-air and wave-crest potentials over the scene's
 * grid-sorted particles and cell tables of the last step
 * (spray_emit.wgsl), then per-class simulation of every slot of the ring
 * buffer (spray_simulate.wgsl). Two deliberate differences, both
 * deterministic: a frame's spawns take consecutive ring slots in sorted
 * particle order (the reference takes them with an atomic counter, so its
 * order is unspecified; this is its order when invocations run in index
 * order), and the potential ceilings' running average (spray.rs:40-50) is
 * updated on the device from each frame's maxima and used from the next
 * frame on (the reference reads the maxima back asynchronously, at least
 * one frame late). fs_spray_step ignores params->ta_limit and wc_limit. */
typedef struct FsSpray FsSpray;
int fs_spray_create(FsSim *sim, uint32_t scene, uint32_t max_particles, FsSpray **out);
int fs_spray_destroy(FsSpray *spray);
/* One frame: emit, simulate, update the ceilings. Asynchronous. */
int fs_spray_step(FsSpray *spray, const GpuSprayParams *params);
/* SpraySystem::reset: every slot dead, write head 0, ceilings to their
 * initial 3.0 / 1.0. */
int fs_spray_reset(FsSpray *spray);
/* Live counts after the last frame: total, spray, foam, bubble (synchronises). */
int fs_spray_stats(FsSpray *spray, uint32_t out[4]);
/* The current ceilings (trapped air, wave crest) and write head (synchronises). */
int fs_spray_limits(FsSpray *spray, float limits[2], uint32_t *write_head);
/* The ring buffer's first `count` records (synchronises), or its device
 * address (GpuSprayParticle[max_particles]) for a renderer. */
int fs_spray_download(FsSpray *spray, GpuSprayParticle *out, uint32_t count);
int fs_spray_device_buffer(FsSpray *spray, void **out);

/* ---- read-outs (synchronising) ------------------------------------------- */

/* Canonical particle buffer as the reference's 64-byte AoS (particle_buffer). */
int fs_download_particles(FsSim *sim, SphParticle3D *out, uint32_t count);
/* Grid-sorted particle buffer as 64-byte AoS (sorted_particle_buffer): the
 * record copied at reorder, with density, near_density and normal as written
 * by the density pass. */
int fs_download_sorted(FsSim *sim, SphParticle3D *out, uint32_t count);
/* cell_counts_buffer and cell_starts_buffer (inclusive prefix ends). Either
 * pointer may be NULL. */
int fs_download_cells(FsSim *sim, uint32_t *counts, uint32_t *starts,
                      uint32_t total_cells);
/* particle_cell_indices (orig -> sorted slot after reorder) and
 * sorted_to_orig. Either pointer may be NULL. */
int fs_download_index_maps(FsSim *sim, uint32_t *cell_indices,
                           uint32_t *sorted_to_orig, uint32_t count);
/* The same 64-byte records written into DEVICE memory, asynchronously on the
 * simulation's stream (the AoS vertex buffer a renderer instances from,
 * particle_renderer_3d.rs:144-160: position at offset 0, velocity at 16):
 * scene `scene`'s canonical particles [0, count) (sorted = 0, the
 * particle_buffer view) or its sorted slots [0, count) (sorted != 0, the
 * sorted_particle_buffer view). device_out is CUDA device (on the
 * simulation's GPU) or managed memory, 16-byte aligned, count * 64 bytes;
 * anything else returns FS_E_INVALID_ARGUMENT. */
int fs_export_particles_aos(FsSim *sim, uint32_t scene, int sorted, SphParticle3D *device_out,
                            uint32_t count);
/* Overwrite the canonical particle records (all fields) of [0, count). */
int fs_upload_particles(FsSim *sim, const SphParticle3D *particles,
                        uint32_t count);

/* The marching-cubes density pass, mc_density.wgsl:130-231 (dispatched at
 * src/render/marching_cubes.rs:2462-2468), in its isotropic form (anisotropy
 * off): the poly6 density (no mass factor) at the centres of grid_size^3
 * voxels, x fastest, summed over the particles of the SPH cells within
 * ceil(kernel_radius / cell) of the voxel's cell, from the grid-sorted
 * positions and cell tables of the scene's last step (the buffers the
 * reference binds). With geom->clip_enabled, voxels outside the box hold -1;
 * the others are divided by the five-wall boundary gamma (floor 0.15).
 * pow(h, 9) is binary exponentiation in double rounded once to float (WGSL
 * leaves pow's precision to the implementation). `density` receives the
 * field: host memory (synchronises) or, with density_on_device != 0, device
 * memory (asynchronous on the simulation's stream). grid_size <= 1024.
 * `scene` is 0 for a plain simulation. */
int fs_density_splat(FsSim *sim, uint32_t scene, const GpuMcGridParams *grid,
                     const GpuContainerGeometry *geom, float *density,
                     int density_on_device);

/* Borrow device memory zero-copy (buffer getters). */
int fs_device_pointers(FsSim *sim, FsDevicePointers *out);
/* Launch on a caller-provided cudaStream_t from now on (NULL = own stream). */
int fs_set_stream(FsSim *sim, void *cuda_stream);
/* Wait for all queued work; reports a device-side wait timeout if one fired. */
int fs_sync(FsSim *sim);

/* ---- per-stage timing ---------------------------------------------------- */

#define FS_STAGE_COUNT 10
/* Stage ids for fs_stage_times: 0 clear, 1 hash, 2 scan, 3 reorder,
 * 4 density, 5 xsph, 6 force+predict, 7 pcisph solve (all iterations),
 * 8 finalize+integrate, 9 whole step. */
/* Enable CUDA-event timing of every stage of subsequent fs_step calls (graph
 * replay is disabled while enabled). */
int fs_enable_stage_timing(FsSim *sim, int enable);
/* Accumulated milliseconds per stage and the number of timed steps since the
 * last reset; synchronises. */
int fs_stage_times(FsSim *sim, double ms[FS_STAGE_COUNT], uint32_t *steps,
                   int reset);
/* Neighbour statistics accumulated by the steps since the last reset (the
 * FLOP model's inputs, measured from the data): out[0] candidate pair tests
 * of the density pass (also the XSPH and force passes' candidates), out[1]
 * density-pass pairs with r^2 < h^2 (self included), out[2] pairs with
 * 1e-12 < r^2 < h^2 (XSPH/force hits), out[3] candidate tests summed over all
 * PCISPH solve iterations, out[4] solve pairs with r^2 < h^2, out[5] particles
 * whose force pass ran cooperatively (a warp on one heavy particle; summed
 * over steps). Synchronises. */
#define FS_STAT_COUNT 6
int fs_neighbor_stats(FsSim *sim, uint64_t out[FS_STAT_COUNT], int reset);

/* ---- batched form ----------------------------------------------------------- */

/* No counterpart in the reference, whose App owns one SphSimulation3DGrid
 * (src/app.rs:253). A batch is a simulation holding independent scenes, each
 * with its own particles, SphParams, container (box, tilt), gravity, mouse
 * force, rigid body and grid (fs_grid_params_for of its kernel radius and
 * count), stepped together: every stage is one launch over all scenes, and
 * scene k's results are bit for bit those of fs_create on the same inputs.
 * The simulation-wide calls (fs_step, fs_prepare_steps, fs_set_pcisph_iterations,
 * fs_clear_rigid_body_accum (all scenes), fs_num_particles (all scenes),
 * fs_device_pointers, fs_set_stream, fs_sync, the timing and statistics
 * calls, fs_destroy) take a batch; the per-scene plain calls return
 * FS_E_STATE on a batch of more than one scene, and fs_spawn_particles is
 * not available for batches. */
#define FS_BATCH_MAX_SCENES 65535u

/* Where scene k lives in the batch's device arrays (fs_device_pointers):
 * canonical particles [particle_offset, particle_offset + num_particles),
 * sorted slots [sorted_offset, sorted_offset + active_particles), cells
 * [cell_offset, cell_offset + total_cells); the cell_starts/cell_begin
 * entries of its cells count slots from 0, not from sorted_offset. */
typedef struct FsSceneInfo {
    uint32_t particle_offset;
    uint32_t num_particles;
    uint32_t active_particles; /* min(params.num_particles, num_particles) */
    uint32_t sorted_offset;
    uint32_t cell_offset;
    uint32_t total_cells;
    uint32_t _pad[2];
    GpuGridParams grid;        /* the scene's grid (num_particles = active) */
} FsSceneInfo;

/* particles: all scenes' records, scene after scene; scene_counts,
 * params and geoms: one entry per scene. Each scene starts with the
 * defaults of fs_create (gravity (0,-9.8,0), mouse force and rigid body
 * inactive). The SDF is shared by all scenes. */
int fs_batch_create(const SphParticle3D *particles, const uint32_t *scene_counts,
                    uint32_t num_scenes, const GpuSphParams3D *params,
                    const GpuContainerGeometry *geoms, const float *sdf,
                    uint32_t sdf_res, int device, uint32_t abi_version,
                    FsSim **out);
int fs_batch_num_scenes(const FsSim *sim, uint32_t *out);
int fs_batch_scene_info(const FsSim *sim, uint32_t scene, FsSceneInfo *out);
/* The update_* uploads for one scene; NULL arguments keep their value. */
int fs_batch_update_scene(FsSim *sim, uint32_t scene, const GpuSphParams3D *params,
                          const GpuContainerGeometry *geom, const GpuGravity *gravity,
                          const GpuMouseForce *mouse, const GpuRigidBody *body);
/* Accumulators of scenes [0, num_scenes); synchronises. */
int fs_batch_read_rigid_body_accum(FsSim *sim, GpuRigidBodyAccum *out,
                                   uint32_t num_scenes);
/* Per-scene read-outs and upload, in scene-local numbering (synchronising). */
int fs_batch_download_scene(FsSim *sim, uint32_t scene, SphParticle3D *out,
                            uint32_t count);
int fs_batch_download_scene_sorted(FsSim *sim, uint32_t scene, SphParticle3D *out,
                                   uint32_t count);
int fs_batch_download_scene_cells(FsSim *sim, uint32_t scene, uint32_t *counts,
                                  uint32_t *starts, uint32_t total_cells);
int fs_batch_download_scene_index_maps(FsSim *sim, uint32_t scene,
                                       uint32_t *cell_indices,
                                       uint32_t *sorted_to_orig, uint32_t count);
int fs_batch_upload_scene(FsSim *sim, uint32_t scene, const SphParticle3D *particles,
                          uint32_t count);

/* ---- differentiable rollout (reverse mode) ------------------------------------ */

/* No counterpart in the reference. Gradients of a rollout of fs_step with
 * respect to the initial canonical positions and velocities and to each
 * scene's viscosity, stiffness and surface_tension, the counterpart of a
 * torch.autograd.Function: fs_adj_forward records, fs_adj_backward consumes
 * cotangents of the final state. Cell assignment and neighbour sets are
 * piecewise constant (taken from the recorded steps, not differentiated); the
 * r < 0.1h fallback direction is constant. The forward keeps the state every
 * `checkpoint_every` steps; the backward recomputes each segment from its
 * checkpoint, recording the step intermediates, and reverses it (segments
 * whose tape the forward recorded are reversed directly). Per-particle
 * adjoints are FP32; the parameter gradients are reduced in FP64 (stiffness
 * is read by no stage of the step: its gradient is 0). Supported: every
 * particle active, mouse force and rigid body inactive, at most 16 PCISPH
 * iterations, every particle inside the SPH grid (else fs_adj_backward
 * returns FS_E_STATE). Works on plain simulations and batches. */
typedef struct FsAdj FsAdj;
/* An FsAdj (like an FsSpray) refers to its simulation: destroy it first. */
int fs_adj_create(FsSim *sim, uint32_t checkpoint_every, FsAdj **out);
int fs_adj_destroy(FsAdj *adj);
/* Run nsteps steps from the simulation's current state, recording; the
 * cotangents are cleared. The parameters must not change until the
 * backward. The last checkpoint segment's tape is recorded on the way (and,
 * with a tape budget, the last S segments'), so the backward re-runs only
 * the other segments. */
int fs_adj_forward(FsAdj *adj, uint32_t nsteps);
/* Device memory the tape may take, in bytes (default 0: one segment of
 * `checkpoint_every` steps). From the next fs_adj_forward on, the tape
 * holds S = min(budget / segment bytes, segments of the rollout) segments
 * (at least 1), recorded during the forward and reversed without re-running
 * them; checkpoints are still kept every `checkpoint_every` steps and the
 * earlier segments re-run from them. If the S buffers cannot be allocated
 * the tape falls back to one segment until the budget is set again. */
int fs_adj_set_tape_budget(FsAdj *adj, uint64_t bytes);
/* Tape segments allocated by the last fs_adj_forward (0 before any) and the
 * bytes one segment takes. Either pointer may be NULL. */
int fs_adj_tape_info(FsAdj *adj, uint32_t *segments, uint64_t *segment_bytes);
/* Cotangents dL/dpos and dL/dvel of the final canonical state, (N, 3) float
 * rows (N = fs_num_particles), host or device memory; NULL = zero. */
int fs_adj_set_cotangents(FsAdj *adj, const float *dl_dpos, const float *dl_dvel,
                          int on_device);
/* A loss as cotangent source: the mean squared difference between the
 * density splat (fs_density_splat) of the scene's final positions and
 * `target` (grid_size^3 floats, host or device). Writes the loss and sets
 * the cotangents of that scene's particles (velocity cotangent 0). */
int fs_adj_splat_mse_loss(FsAdj *adj, uint32_t scene, const GpuMcGridParams *grid,
                          const GpuContainerGeometry *geom, const float *target,
                          int target_on_device, double *loss);
/* No counterpart in the reference. fs_adj_splat_mse_loss for `count` scenes
 * at once (scenes[k] with grids[k], geoms[k] and targets[k], all targets on
 * the host or all on the device): the final positions are grid-sorted once
 * and the losses are read back once, into losses[0 .. count). Losses and
 * cotangents are those of the single-scene calls. */
int fs_adj_splat_mse_losses(FsAdj *adj, uint32_t count, const uint32_t *scenes,
                            const GpuMcGridParams *grids, const GpuContainerGeometry *geoms,
                            const float *const *targets, int targets_on_device,
                            double *losses);
/* The density splat (fs_density_splat) of the scene's FINAL positions after
 * fs_adj_forward, e.g. to build a target field from a hidden run: host or
 * device memory, grid_size^3 floats. */
int fs_adj_final_splat(FsAdj *adj, uint32_t scene, const GpuMcGridParams *grid,
                       const GpuContainerGeometry *geom, float *out, int out_on_device);
/* Reverse the recorded rollout: dL/dpos0 and dL/dvel0 as (N, 3) float rows
 * (host or device, either may be NULL) and, if dl_dparams is not NULL,
 * 3 doubles per scene (viscosity, stiffness, surface_tension). Leaves the
 * simulation at the rollout's final canonical state (its sorted views are
 * unspecified until the next step). Synchronises. */
int fs_adj_backward(FsAdj *adj, float *dl_dpos0, float *dl_dvel0, int on_device,
                    double *dl_dparams);
/* No counterpart in the reference. The scalar-parameter gradients of the
 * last fs_adj_backward, FS_ADJ_NUM_PARAMS doubles per scene (`scenes` must be
 * the simulation's scene count), in the order viscosity, stiffness,
 * surface_tension, near_stiffness, pcisph_delta. stiffness is read by no
 * stage of the step (pressure strength comes from pcisph_delta,
 * pcisph_solve.wgsl:178-179), so its gradient is 0; near_stiffness scales the
 * near pressure of sph_force_3d_grid.wgsl:127, 180-183 and pcisph_delta the
 * pressure update of pcisph_solve.wgsl:178-179. Each per-particle share is
 * FP32 and the sums are FP64. */
#define FS_ADJ_NUM_PARAMS 5
int fs_adj_param_gradients(FsAdj *adj, double *out, uint32_t scenes);

/* ---- prefix scan without allocation -------------------------------------- */

/* No counterpart in the reference. The inclusive prefix scan of a cell-count
 * array (the reference's cell_starts, prefix_scan.wgsl) for callers that
 * cannot allocate device memory: code inside a CUDA stream capture that must
 * not add allocation nodes, real-time loops that forbid allocator calls and
 * their implicit synchronisation after start-up, and hosts whose device
 * memory is owned by another runtime. It allocates nothing: the scan's tile
 * descriptors live in a fixed file-scope device array of 128 KiB that every
 * GPU loading the library holds until the process exits. cell_counts and
 * cell_starts are device arrays of total_cells entries, at most
 * FS_NOALLOC_SCAN_MAX_CELLS (larger sizes return FS_E_CAPACITY).
 * device_status, if not NULL, is a device word the kernel ORs 1 into if its
 * bounded look-back wait ever gives up. Asynchronous on `stream` (a
 * cudaStream_t, NULL = legacy default stream). All calls share the array:
 * each clears it on its stream first, but calls that overlap on the GPU race.
 * The first call on a device looks up the array's address (with that device
 * current); make it before any stream capture. Later calls outside a capture
 * look the address up again, so a rebuilt context is followed. */
#define FS_NOALLOC_SCAN_MAX_CELLS (1u << 26)
int fs_prefix_scan_noalloc(const uint32_t *cell_counts, uint32_t *cell_starts,
                           uint32_t total_cells, uint32_t *device_status,
                           void *stream);

/* ---- failure-detection self-test ------------------------------------------
 * No counterpart in the reference (its prefix scan has no waits across
 * workgroups). Exercises the bounded look-back wait of the prefix scan the
 * step runs (decoupled look-back, prefix_scan.wgsl's role) and its reporting
 * path. Runs that scan over the simulation's current cell counts into scratch
 * of its own (the simulation's tables are left as they are). With inject != 0
 * every look-back polls a descriptor that nothing publishes and gives up
 * after a short bound, as a wait that ran out would: the kernel still
 * finishes (with a wrong prefix) and records the expiry in the simulation's
 * device error word, so the next synchronising call (fs_sync,
 * fs_read_rigid_body_accum, the downloads) returns FS_E_DEVICE_TIMEOUT and
 * clears the word; the call after that returns FS_OK. With inject = 0 the
 * result equals the step's cell_starts. starts_out (host, total cells), if
 * not NULL, receives the scan's output. Synchronises the simulation's stream
 * without reading the error word. */
int fs_selftest_scan_wait(FsSim *sim, int inject, uint32_t *starts_out);

/* ---- arithmetic self-test ---------------------------------------------------
 * No counterpart in the reference. The force and solve passes compute square
 * roots, reciprocals and quotients from the hardware approximations
 * (rsqrt.approx, rcp.approx) refined to the correctly rounded result, where
 * every operand of a pair lies in [2^-60, 2^60), and with the IEEE operations
 * otherwise; the results are the IEEE bits. This call re-checks that on
 * `device`: results[0] = bit patterns (all 2^32) whose reciprocal differs
 * from __frcp_rn, [1] = the same for the square root against sqrtf, [2] =
 * quotients that differ from IEEE division on 2^32 pseudo-random operand pairs
 * (half of them inside the fast range), [3] = how many of those pairs took the
 * fast path. The first three are 0 on a device the library's parity claims
 * hold for. Synchronous, tens of milliseconds. */
int fs_selftest_arithmetic(int device, unsigned long long results[4]);

/* No counterpart in the reference. Measured FP32 pipe throughput of
 * `device`, the denominator of the neighbour passes' FP32 roofline:
 * tflops[0] = fused multiply-add (2 FLOP per instruction), tflops[1] =
 * separate multiply and add (the non-contracted arithmetic that bit-exact
 * kernels compile to). Each is the best of five timed launches of eight
 * independent dependency chains per thread at 32 warps per SM. Synchronous,
 * about 0.2 s. */
int fs_selftest_fp32_rate(int device, double tflops[2]);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* FLUIDSPH_H */
