/*
 * suna.h — C ABI of the GB300 engine for SunaEngine's deterministic Q16.16
 * position-based-fluids substep.
 *
 * This is the boundary a host binds (a Node N-API addon, ctypes, cgo ...). It
 * replaces the `Engine` object of the reference's `src/engine.js`
 * (createEngine at src/engine.js:2786, class Engine at src/engine.js:3523) and
 * the per-scene calls its demo layer makes (src/demo_boot.js:71-420).
 *
 * Conventions
 *   - plain pointers and sizes only; the caller owns every host buffer and the
 *     engine copies in and out;
 *   - every call returns an int status: SN_OK (0) or a negative SN_E_* code;
 *     sn_last_error() gives the message (the reference throws
 *     Error('[aether] ...') synchronously, src/engine.js:2174);
 *   - one engine = one CUDA stream on one GPU; an engine is not re-entrant and
 *     must be driven from one host thread at a time (the reference's engine is
 *     single-threaded JS);
 *   - GPU-side failures are deferred and reported by sn_check_errors(), like
 *     the reference's checkErrors() (src/engine.js:3689-3696).
 *
 * State words are the reference's Particle struct (src/sim.wgsl:181-188):
 * 8 int32 per particle, [pos.x, pos.y, vel.x, vel.y, matId, flags, temp, fuel],
 * in slot order: fluid slots [0, nFluid), then the boundary block.
 */
#ifndef SUNA_H
#define SUNA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SN_OK 0
#define SN_E_INVALID (-1)      /* a bad argument: the reference's assert() */
#define SN_E_CAPACITY (-2)     /* does not fit the capacities given at create */
#define SN_E_UNSUPPORTED (-3)  /* a material row whose passes this engine does not run */
#define SN_E_CUDA (-4)         /* a CUDA runtime error */
#define SN_E_STATE (-5)        /* called in the wrong state (e.g. step before load) */
#define SN_E_DEVICE (-6)       /* the device reported an error word (see sn_check_errors) */

typedef struct sn_engine sn_engine;

/* createEngine options (src/engine.js:2786-2820). */
typedef struct sn_opts {
  uint32_t max_particles; /* slot capacity (maxParticles) */
  uint32_t max_cells;     /* grid-cell capacity (maxCells); 0 = 1<<20 */
  uint32_t iters;         /* solver iterations, 1..16 (ITERS = 4, src/engine.js:245) */
  uint32_t debug;         /* 1 = count fp_flag events into the 16 debug words */
  uint32_t chain;         /* 1 = fold every substep's digest into the chain */
  int32_t device;         /* CUDA device ordinal */
  const int32_t* luts;    /* 5*3202 int32 kernel tables (src/tables.json), hash-checked */
  const int32_t* mats;    /* mat_count rows of 48 int32 (MATS, src/engine.js:1192) */
  uint32_t mat_count;     /* 1..64 */
  uint32_t lanes;         /* lanes per particle in the neighbour gathers: 1, 2, 4, 8;
                             0 = chosen from the active particle count. Results do
                             not depend on it (the split sums are exact). */
} sn_opts;

/* loadScene argument (src/engine.js:3704-3951). flags/temp/fuel may be NULL. */
typedef struct sn_scene {
  uint32_t n, n_fluid;
  const int32_t* pos;     /* 2n */
  const int32_t* vel;     /* 2n */
  const uint32_t* mat_id; /* n */
  const uint32_t* flags;  /* n or NULL */
  const int32_t* temp;    /* n or NULL */
  const int32_t* fuel;    /* n or NULL */
  int32_t dom_w, dom_h;   /* ticks */
  uint32_t cell_shift;    /* 18 = 4 wu cells */
} sn_scene;

/* One spawned particle (spawnFluid list entry, src/engine.js:5901). */
typedef struct sn_particle {
  int32_t x, y, vx, vy;
  int32_t mat;
  uint32_t flags;         /* only FLAG_BURNING | FLAG_ANCHOR are taken */
  int32_t temp, fuel;
  uint32_t has_temp, has_fuel; /* 0 = the material's spawnTemp / fuel0 */
} sn_particle;

typedef struct sn_info {
  uint32_t n, n_fluid;
  uint64_t substep_count;
  uint64_t formation_clock;
  uint32_t grid_w, grid_h, cell_total;
} sn_info;

/* ---- single-scene engine: the drop-in for engine.js's Engine ------------- */

/* createEngine (src/engine.js:2786). */
int sn_create(const sn_opts* opts, sn_engine** out);
/* destroy (src/engine.js Engine.destroy). */
void sn_destroy(sn_engine* e);
/* Text of the last error on this engine (valid until the next call). */
const char* sn_last_error(const sn_engine* e);
/* Engine.loadScene (src/engine.js:3704). Resets the chain and the clocks. */
int sn_load_scene(sn_engine* e, const sn_scene* scene);
/* Engine.step (src/engine.js:3963): advance exactly `count` substeps. Encodes
 * asynchronously; returns the new substep count in *substeps (may be NULL). */
int sn_step(sn_engine* e, uint32_t count, uint64_t* substeps);
/* Engine.digest (src/engine.js:4453): H_set (acc[0..3]) || H_slot (acc[4..7])
 * of the current state. Synchronous. */
int sn_digest(sn_engine* e, uint32_t acc[8]);
/* Engine.chainHex (src/engine.js:4406): the folded per-substep chain. */
int sn_chain(sn_engine* e, uint32_t chain[8]);
/* Engine.resetChain (src/engine.js:3953). */
int sn_reset_chain(sn_engine* e);
/* Engine.readState: n*8 words of the current state. */
int sn_read_state(sn_engine* e, int32_t* out, size_t words);
/* The positions the last loadScene loaded (2 words per particle of that load:
 * the engine's _initialPos, src/engine.js:3947, kept on the device; spawns
 * and edits do not change it). *words_out receives the word count. */
int sn_read_initial_positions(sn_engine* e, int32_t* out, size_t words, size_t* words_out);
/* The cross-substep scratch an exact keyframe needs: stAcc, n*2 words
 * (Derived.stAcc, src/sim.wgsl:200; consumed by predict at src/sim.wgsl:980). */
int sn_read_scratch(sn_engine* e, int32_t* out, size_t words);
/* Exact keyframe restore (WaterDemo.restore, src/demo_boot.js:308-320): the
 * state words (n*8) and optionally the scratch (n*2, NULL = zero, i.e. a load
 * boundary). The scene must already be loaded with the same n / nFluid. */
int sn_write_state(sn_engine* e, const int32_t* state, const int32_t* scratch, size_t n);
/* Bond rows, nFluid*48 packed words (src/sim.wgsl:1594-1617). */
int sn_read_bonds(sn_engine* e, uint32_t* out, size_t words);
/* The last substep's per-slot fields that Engine.liveness (src/engine.js:
 * 4490-4511) reads: the rho column of readDerived (:4290, Derived.rho,
 * src/sim.wgsl:200) and the neighbour count of readNbrN (:4291; the count
 * field only, without the reference's seal/congeal flag bits), n words each
 * in slot order, 0 for wall slots; either pointer may be NULL. SN_E_INVALID
 * when no substep has run since the particles last changed (load, spawn,
 * erase, state write, checkpoint load). */
int sn_read_fields(sn_engine* e, int32_t* rho, uint32_t* nbr_count, size_t n);
/* Engine.readCellStart (src/engine.js:4292): cell_total + 1 words in the
 * reference's layout, as of the last substep's grid: entry c (row-major cell
 * index cy*gridW + cx) is the first position of cell c in a sort by cell
 * index, entry cell_total the particle count. (This engine's own sorted order
 * is tile-major; the entries are rebuilt from its per-cell occupancies.) Same
 * refusal as sn_read_fields. */
int sn_read_cell_start(sn_engine* e, uint32_t* out, size_t words);
/* Engine.spawnFluid (src/engine.js:5901): append k fluid particles, relocate
 * the boundary block to the tail. *n_out = new n (unchanged when the capacity
 * refuses, as the reference silently does). `no_weld` holds the options bits:
 * SN_SPAWN_NO_WELD ({noWeld: true}: no weld tag), SN_SPAWN_OWN_GROUP
 * ({ownGroup: true}: its own group even while a gesture is held). */
#define SN_SPAWN_NO_WELD 1u
#define SN_SPAWN_OWN_GROUP 2u
int sn_spawn(sn_engine* e, const sn_particle* list, uint32_t k, uint32_t no_weld, uint32_t* n_out);
/* Weld groups (src/engine.js:4570-4680): beginWeldGroup opens a gesture (every
 * spawn joins it until endWeldGroup) and returns its tag; holdWeldGroup holds
 * an existing tag; endWeldGroup releases (formation runs on the next
 * substep); armFuse arms draw-time fusion (§18.24) for the open gesture, and
 * the arm is cleared by the first sn_step after the release.
 * sn_weld_state: {weldHold, fuseTag, lastWeldTag, weldSeq}. */
int sn_begin_weld_group(sn_engine* e, uint32_t* tag);
int sn_hold_weld_group(sn_engine* e, uint32_t tag);
int sn_end_weld_group(sn_engine* e, uint32_t* was);
int sn_arm_fuse(sn_engine* e, uint32_t* tag);
int sn_weld_state(sn_engine* e, uint32_t out[4]);
/* Engine.applyImpulse (src/engine.js:6077): add (ix, iy) to the velocity of the
 * first `limit` fluid particles in slot order within r of (cx, cy), clamped to
 * +-VMAX. Applied on the device at the current substep boundary. */
int sn_impulse(sn_engine* e, int32_t cx, int32_t cy, int32_t r, int32_t ix, int32_t iy, uint32_t limit,
               uint32_t* hits);
/* Engine.debugCounters: the 16 fp_flag words (zero unless opts.debug). */
int sn_debug_counters(sn_engine* e, uint32_t out[16]);
/* Engine.checkErrors: SN_OK, SN_E_CUDA or SN_E_DEVICE. */
int sn_check_errors(sn_engine* e);
/* Block until all queued work is done. */
int sn_sync(sn_engine* e);
int sn_get_info(sn_engine* e, sn_info* out);
/* Engine.setWalls (src/engine.js:5262): take the scene's boundary block out
 * (n = nFluid) or rewrite it from the loaded scene and put it back. */
int sn_set_walls(sn_engine* e, uint32_t on, uint32_t* walls_on);
/* Formation clock and pending-formation flag (engine `_substep`, `_bondDirty`),
 * for keyframes that must resume the bond-formation schedule exactly. */
int sn_set_formation_clock(sn_engine* e, uint64_t clock, uint32_t dirty);

/* ---- batched engine: many independent scenes, one launch sequence -------- */
/* No counterpart in the reference (which runs one scene per engine); the
 * per-scene semantics are exactly the single engine's. */

typedef struct sn_batch sn_batch;

/* opts->max_particles is the total slot capacity over all scenes. */
int sn_batch_create(const sn_opts* opts, uint32_t max_scenes, sn_batch** out);
void sn_batch_destroy(sn_batch* b);
const char* sn_batch_last_error(const sn_batch* b);
/* Add a scene with `capacity` slots (>= scene->n; room for spawns). */
int sn_batch_add_scene(sn_batch* b, const sn_scene* scene, uint32_t capacity, uint32_t* id);
/* Drop a scene; its slots are reused by later adds of the same or smaller size. */
int sn_batch_remove_scene(sn_batch* b, uint32_t id);
/* Advance every scene by `count` substeps. */
int sn_batch_step(sn_batch* b, uint32_t count);
/* Queue a disc impulse for scene `id`, applied before that scene's substep
 * number `at_substep` (counted from its load) runs. Events of one scene must be
 * queued in nondecreasing at_substep; same-substep events apply in queue order. */
int sn_batch_schedule_impulse(sn_batch* b, uint32_t id, uint64_t at_substep, int32_t cx, int32_t cy,
                              int32_t r, int32_t ix, int32_t iy, uint32_t limit);
int sn_batch_digest(sn_batch* b, uint32_t id, uint32_t acc[8]);
int sn_batch_chain(sn_batch* b, uint32_t id, uint32_t chain[8]);
int sn_batch_read_state(sn_batch* b, uint32_t id, int32_t* out, size_t words);
int sn_batch_read_scratch(sn_batch* b, uint32_t id, int32_t* out, size_t words);
int sn_batch_write_state(sn_batch* b, uint32_t id, const int32_t* state, const int32_t* scratch, size_t n,
                         uint64_t substep_count, uint64_t formation_clock, uint32_t dirty);
int sn_batch_get_info(sn_batch* b, uint32_t id, sn_info* out);
int sn_batch_check_errors(sn_batch* b);
int sn_batch_sync(sn_batch* b);
/* Device time of the last sn_batch_step / sn_step in milliseconds (CUDA
 * events on the engine's stream), and the kernel launches it issued. */
int sn_batch_last_timing(sn_batch* b, float* ms, uint64_t* launches);
int sn_last_timing(sn_engine* e, float* ms, uint64_t* launches);
/* profileSubstep (src/engine.js:4221-4267): run `reps` substeps (outside the
 * CUDA graph) with CUDA events between kernel phases and return the mean
 * device milliseconds of each phase in ms[0..*n_phases). Phase order:
 * predict, grid sort, cell ranges + gather, neighbour lists, then per solver
 * iteration (solveA, the four colour passes, friction), then
 * finalize/xsph/normals/conduct, surface tension/thermal/formation/digest,
 * chain fold. The substeps are real: the scene advances by `reps`. */
int sn_profile_substep(sn_engine* e, uint32_t reps, float* ms, uint32_t max_phases, uint32_t* n_phases);
int sn_batch_profile_substep(sn_batch* b, uint32_t reps, float* ms, uint32_t max_phases, uint32_t* n_phases);

/* ---- authoring edits -----------------------------------------------------------
 * The device halves of the reference's host-side edits (src/engine.js:
 * replaceWhere :6191, sliceBondsMany :6240, eraseWhere :6460): the caller
 * evaluates its predicate on a readState copy, as the reference does in JS.
 * sn_write_bonds writes nFluid*48 bond words (replaceWhere / sliceBonds
 * tombstone bonds on the host and write the rows back; call
 * sn_set_formation_clock(..., dirty = 1) after, as they set _bondDirty).
 * sn_erase keeps the fluid slots whose keep[i] != 0 (n = nFluid flags):
 * survivors stay in order, the boundary block follows them, stAcc moves with
 * its particle, bond partners are renumbered and bonds to erased particles
 * (and tombstones) are dropped, and formation runs on the next substep;
 * *removed receives the count. */
int sn_write_bonds(sn_engine* e, const uint32_t* bonds, size_t words);
int sn_batch_write_bonds(sn_batch* b, uint32_t id, const uint32_t* bonds, size_t words);
int sn_erase(sn_engine* e, const uint8_t* keep, size_t n, uint32_t* removed);
int sn_batch_erase(sn_batch* b, uint32_t id, const uint8_t* keep, size_t n, uint32_t* removed);

/* ---- inputs: jets and the user drive ------------------------------------------
 * setJets (src/engine.js:4740-4770): up to 8 jets per scene, [x, y, r, fx, fy]
 * int32 each (ticks; fx/fy in the units of Mat.grav); extra entries are
 * ignored, as the reference slices to JET_MAX. A particle whose position lies
 * in a jet's disc gets its acceleration in predict (jet_accel,
 * src/sim.wgsl:935-949). k = 0 removes them (bit-inert). *n_out = jets kept.
 * setUserDrive (src/engine.js:4797-4815) is stored clamped to +-USER_A_MAX
 * (32768) and returned in out[2]; rigidStep adds it to the velocity of every
 * free body flagged as the user's (RB_USER). */
int sn_set_jets(sn_engine* e, const int32_t* jets, uint32_t k, uint32_t* n_out);
int sn_batch_set_jets(sn_batch* b, uint32_t id, const int32_t* jets, uint32_t k, uint32_t* n_out);
int sn_set_user_drive(sn_engine* e, int32_t ax, int32_t ay, int32_t out[2]);

/* ---- §20 rigid bodies (src/sim.wgsl:3070-3747; host src/engine.js:5452-5811) ---
 * A body is a set of fluid slots of a solidMode-rigid row wearing FLAG_RIGID
 * and one weld tag; its record (32 int32 words, the reference's RB_* layout,
 * src/sim.wgsl:703-793) holds centre, velocity, angle (BAM), spin, carried
 * remainders, member count and inertia; every member is placed at
 * c + R(theta) * o each substep from its exact rest offset o.
 *   sn_make_rigid_body   makeRigidBody(slots, pivot, user) :5722 (pivot NULL:
 *                        a free body; {x, y} ticks: an axis body, makeAxisBody)
 *   sn_promote_weld_group promoteWeldGroup(tag, pivot, user) :5584 (tag 0 =
 *                        the gesture held open)
 *   sn_end_weld_group_and_promote endWeldGroupAndPromote(pivot, user) :5782
 *   sn_dissolve_all_bodies dissolveAllBodies() :5789, *count = members freed
 *   sn_read_bodies       readBodies() :5811: *count records of 32 words (word
 *                        29 reads 0); out may be NULL to get the count
 *   sn_read_rest_offsets readRestOffsets() :5817: n*2 words
 *   sn_set_body_user     setBodyUser(index, on) :5319
 *   sn_set_body_driver   one body's driver sidecar (the words
 *                        setBodyConstraint's evaluator uploads, :5343-5412):
 *                        mask of RD_HAS_* bits (< 512) and nine values
 *                        {px, py, angle, vx, vy, omega, fx, fy, torque}; they
 *                        hold until changed or cleared
 *   sn_drag_body         dragGrab(grab, x, y, vx, vy) for a rigid grab :6111
 *   sn_restore_bodies    restoreAuthoringSnapshot's body records and rest
 *                        offsets :5838 (drivers cleared)
 * Index arguments and *index results are the body's position in readBodies;
 * *index = -1 where the reference returns null (too few members, no slot).
 * eraseWhere repairs the bodies (survivors keep their rest offsets); a scene
 * load dissolves them; a device checkpoint carries them. */
int sn_make_rigid_body(sn_engine* e, const uint32_t* slots, uint32_t k, const int32_t* pivot, uint32_t user,
                       int32_t* index);
int sn_promote_weld_group(sn_engine* e, uint32_t tag, const int32_t* pivot, uint32_t user, int32_t* index);
int sn_end_weld_group_and_promote(sn_engine* e, const int32_t* pivot, uint32_t user, int32_t* index);
int sn_dissolve_all_bodies(sn_engine* e, uint32_t* count);
int sn_read_bodies(sn_engine* e, int32_t* out, size_t words, uint32_t* count);
int sn_read_rest_offsets(sn_engine* e, int32_t* out, size_t words);
int sn_set_body_user(sn_engine* e, uint32_t index, uint32_t on, uint32_t* found);
int sn_set_body_driver(sn_engine* e, uint32_t index, int32_t mask, const int32_t values[9]);
int sn_clear_body_drivers(sn_engine* e);
int sn_drag_body(sn_engine* e, uint32_t tag, int32_t x, int32_t y, int32_t vx, int32_t vy, uint32_t* moved);
int sn_restore_bodies(sn_engine* e, const int32_t* records, uint32_t count, const int32_t* rest, size_t rest_words);
/* The body calls above on scene `id` of a batch (same arguments and results;
 * body indices count that scene's bodies only). Removing the scene, or a
 * load into it, drops its bodies; a device checkpoint carries them. */
int sn_batch_make_rigid_body(sn_batch* b, uint32_t id, const uint32_t* slots, uint32_t k, const int32_t* pivot,
                             uint32_t user, int32_t* index);
int sn_batch_promote_weld_group(sn_batch* b, uint32_t id, uint32_t tag, const int32_t* pivot, uint32_t user,
                                int32_t* index);
int sn_batch_dissolve_all_bodies(sn_batch* b, uint32_t id, uint32_t* count);
int sn_batch_read_bodies(sn_batch* b, uint32_t id, int32_t* out, size_t words, uint32_t* count);
int sn_batch_read_rest_offsets(sn_batch* b, uint32_t id, int32_t* out, size_t words);
int sn_batch_set_body_user(sn_batch* b, uint32_t id, uint32_t index, uint32_t on, uint32_t* found);
int sn_batch_set_body_driver(sn_batch* b, uint32_t id, uint32_t index, int32_t mask, const int32_t values[9]);
int sn_batch_clear_body_drivers(sn_batch* b, uint32_t id);
int sn_batch_drag_body(sn_batch* b, uint32_t id, uint32_t tag, int32_t x, int32_t y, int32_t vx, int32_t vy,
                       uint32_t* moved);
/* _writeBodyRecord (src/engine.js:5452) for host-side rebuilds that choose
 * their members themselves (splitDisconnectedBodies :6313,
 * promoteLooseRigidComponents :5636): members are taken as given, tag 0 draws
 * a fresh tag; FLAG_RIGID and the tag are set on them. *index = -1 below 4
 * members or at 1024 bodies; *tag_out receives the tag used. */
int sn_write_body(sn_engine* e, const uint32_t* members, uint32_t k, uint32_t tag, const int32_t* pivot, uint32_t user,
                  int32_t* index, uint32_t* tag_out);

/* ---- material rows at run time ---------------------------------------------------
 * §25 interned rows (src/engine.js:4981-5245): the host's composition algebra
 * (synth) and intern cache decide a row's 48 words and its row id; the engine
 * only holds the table. sn_set_material writes one row past the authored ones
 * (row == the current count appends; *mat_count receives the new count) with
 * rampInv baked from rampHi - rampLo and grav scaled by the gravity scale, as
 * _internUpload does; sn_clear_materials drops every row past the authored
 * ones (clearInterned). §26.C setGravityScale (src/engine.js:4843): q in Q16,
 * clamped to [0, 4 x 65536]; every row's grav becomes RNE(grav * q / 65536).
 * All three hold for every scene loaded afterwards. */
int sn_set_material(sn_engine* e, uint32_t row, const int32_t words[48], uint32_t* mat_count);
int sn_clear_materials(sn_engine* e);
int sn_set_gravity_scale(sn_engine* e, int32_t q, int32_t* out);
int sn_batch_set_material(sn_batch* b, uint32_t row, const int32_t words[48], uint32_t* mat_count);

/* ---- lane autotuner ----------------------------------------------------------
 * No counterpart in the reference. The neighbour gathers of solveA, the colour
 * passes, post1, post2 and the neighbour-list build can split each particle's
 * list over 1, 2, 4 or 8 lanes; the friction pass takes the colour passes'
 * count. Results are identical for every choice, speed is not. With
 * opts.lanes == 0 each class starts from a rule on the active particle count
 * (re-applied when the scene set changes by more than 2x); sn_autotune runs
 * 4 x (reps + 1) REAL substeps of every loaded scene (the first of each lane
 * count untimed; they advance the scenes and their chains exactly like
 * sn_step) under each lane count with phase timers and keeps the fastest
 * count per class. *substeps_run receives how many substeps it ran. With
 * opts.lanes != 0 the lanes are pinned and it runs none.
 * sn_lanes reports {solveA, colours, post1, post2, neighbour lists}. */
int sn_autotune(sn_engine* e, uint32_t reps, uint32_t* substeps_run);
int sn_batch_autotune(sn_batch* b, uint32_t reps, uint32_t* substeps_run);
int sn_lanes(sn_engine* e, uint32_t out[5]);
int sn_batch_lanes(sn_batch* b, uint32_t out[5]);
/* Pin {solveA, colours, post1, post2, neighbour lists} lanes (each 1, 2, 4 or
 * 8), e.g. a split tuned on another run of the same workload; afterwards
 * neither the size rule nor sn_autotune changes them. */
int sn_set_lanes(sn_engine* e, const uint32_t lanes[5]);
int sn_batch_set_lanes(sn_batch* b, const uint32_t lanes[5]);
/* (no counterpart) The sorted-space layout and gather kernels of solveA and
 * the colour passes. 0 (the default): colour-major sorted space, neighbours
 * gathered from global memory through the neighbour list. 1: tile-major sorted
 * space (4 x 4-cell tiles), each tile's neighbourhood copied into shared memory
 * with bulk copies and gathered there through 16-bit tile-local indices.
 * Results are identical; only speed differs (the staged form measured slower
 * on GB300). Takes effect at the next step. */
int sn_set_staged(sn_engine* e, uint32_t on);
int sn_batch_set_staged(sn_batch* b, uint32_t on);
/* (no counterpart) The staged layout's tiles: 2^shift cells a side, shift 2,
 * 3 or 4 (default 2). Takes effect at the next step. */
int sn_set_tile_shape(sn_engine* e, uint32_t shift);
int sn_batch_set_tile_shape(sn_batch* b, uint32_t shift);
/* (no counterpart) Layout tuning: runs reps + 1 REAL substeps (the first
 * untimed) under each of the list gathers and the staged gathers with tiles
 * of 4, 8 and 16 cells, and keeps the fastest. *substeps_run receives the
 * substeps it ran, *layout the pick (0 = list gathers, else the tile side's
 * log2), ms_per_substep[4] (may be null) the device ms per substep of each
 * candidate in that order. Results are identical under every layout. */
int sn_autotune_layout(sn_engine* e, uint32_t reps, uint32_t* substeps_run, uint32_t* layout, float* ms_per_substep);
int sn_batch_autotune_layout(sn_batch* b, uint32_t reps, uint32_t* substeps_run, uint32_t* layout,
                             float* ms_per_substep);
/* (no counterpart) Run the solver iterations (solveA, the four colour
 * passes and friction/applyFric, ITERS times) as one persistent cooperative
 * kernel with grid barriers between the phases, instead of one launch per
 * phase. Applies to worlds with no rigid body in the default layout; others
 * keep the per-phase launches. Results are identical (measured slower
 * on GB300 than the captured per-phase graph; off by default). A barrier that
 * waits past its bound raises an error that sn_check_errors reports. */
int sn_set_persistent(sn_engine* e, uint32_t on);
int sn_batch_set_persistent(sn_batch* b, uint32_t on);

/* ---- digest without device allocation ------------------------------------ */
/* No counterpart in the reference. For callers that cannot allocate device
 * memory when they need a digest: latency-bound loops that cannot absorb
 * cudaMalloc's device synchronisation, and embedding hosts that own all device
 * memory and forbid libraries from allocating. The caller passes its own
 * device buffers: d_state (n*8 words, the Particle layout above), optionally
 * d_bond (n_fluid*48 packed bond words, or NULL for no bond fold), and d_out
 * (8 words) that receives H_set (0..3) || H_slot (4..7), exactly as sn_digest
 * computes them. Work is queued on `stream` (a cudaStream_t; NULL = the legacy
 * default stream). Scratch is a fixed 64 KiB array in the library's device
 * image, so n is limited to 16,777,216 particles (SN_E_CAPACITY above that,
 * nothing launched). The array is shared by all calls on a device: calls that
 * overlap on the GPU race and must be ordered by the caller. The first call
 * under each CUDA context (per device, and again after cudaDeviceReset or
 * under a context the caller created) looks up the array's device address in
 * that context. */
#define SN_NOALLOC_MAX_PARTICLES 16777216u
int sn_digest_device_noalloc(const int32_t* d_state, uint32_t n, uint32_t n_fluid, const uint32_t* d_bond,
                             uint32_t* d_out, void* stream);

/* ---- 3D solver --------------------------------------------------------------
 * Replaces the simulation half of the reference's 3D page (class App in
 * 3d/app.js: reset :561-568, runSubsteps :709-714, spawn :575-597,
 * setBallRadius :599-604, chain :717-744) and its compute shaders
 * (3d/sim3d.wgsl:188-590). One sn3_engine holds up to max_scenes independent
 * scenes and advances all of them per sn3_step; sn3_load_scene is the
 * single-scene reset() and uses scene 0.
 *
 * State words per particle (slot order): [p.x, p.y, p.z, mat, v.x, v.y, v.z, 0]
 * (the reference's p and v vec4s, 3d/sim3d.wgsl:45-50, with mat in p.w).
 * sn3_fnv returns the reference's own 3D digest (256 FNV-1a stripes folded
 * into 8 lanes, 3d/app.js:717-744); sn3_digest / sn3_chain apply the 2D
 * engine's H_set || H_slot hash to the 8 words above, once per substep into
 * the chain (the reference's 3D page has no per-substep hash; this one has no
 * counterpart there). */
typedef struct sn3_engine sn3_engine;

typedef struct sn3_opts {
  uint32_t max_particles; /* slot capacity over all scenes (the page's NMAX) */
  uint32_t max_cells;     /* grid cells over all scenes; 0 = 1<<20 */
  uint32_t max_scenes;    /* 0 = 1 */
  uint32_t iters;         /* 1..16; the page runs 3 (3d/app.js:21) */
  uint32_t debug;         /* 1 = count fp_flag events into the 16 debug words */
  uint32_t chain;         /* 1 = hash every substep into the chain */
  int32_t device;
  const int32_t* luts;    /* W[2049] | G[2049] | planeW[513] | planeG[513] (buildLUTs, 3d/app.js:85-160) */
  const int32_t* mats;    /* mat_count rows of 4: grav, rhoW, damp, f0 (3d/app.js:180-201) */
  uint32_t mat_count;     /* 1..256; rhoW in -256..3839 */
  uint32_t lanes;         /* lanes per particle in the density and solve gathers: 1, 2 or 4;
                             0 = chosen from the active particle count. Results do not depend
                             on it. */
} sn3_opts;

typedef struct sn3_scene {
  uint32_t n;
  const int32_t* pos;     /* 3n, Q16.16 */
  const int32_t* vel;     /* 3n or NULL (zero) */
  const uint32_t* mat;    /* n */
  uint32_t gx, gy, gz;    /* cells of 2 wu per axis, 1..52 (the page: 28 x 30 x 28) */
  int32_t stir_amp;       /* CFG.stirAmp (3d/app.js:24); 0 = off */
  uint32_t frame;         /* 0: the stir phase is fixed per sn3_step call, as per runSubsteps call in
                             the page; F > 0: fixed per frame of F substeps counted from the load, the
                             same as calling sn3_step(F) repeatedly, whatever the call sizes */
} sn3_scene;

typedef struct sn3_info {
  uint32_t n, cap, gx, gy, gz, iters;
  uint64_t substep_count;
} sn3_info;

int sn3_create(const sn3_opts* opts, sn3_engine** out);
void sn3_destroy(sn3_engine* e);
const char* sn3_last_error(const sn3_engine* e);
/* reset(n, scene) (3d/app.js:561-568): scene 0 with every slot as capacity. */
int sn3_load_scene(sn3_engine* e, const sn3_scene* sc);
/* Add an independent scene with room for `cap` particles (0 = sc->n). */
int sn3_add_scene(sn3_engine* e, const sn3_scene* sc, uint32_t cap, uint32_t* scene_out);
int sn3_remove_scene(sn3_engine* e, uint32_t scene);
/* runSubsteps(count) (3d/app.js:709-714) for every scene; the stir phase is
 * (substepCount * 384) & 131071 at the start of the call, as the page writes
 * its params once per batch. */
int sn3_step(sn3_engine* e, uint32_t count);
/* spawn (3d/app.js:575-597): append k particles (positions in Q16.16, velocity
 * zero); what exceeds the scene's capacity is dropped (*added < k). */
int sn3_spawn(sn3_engine* e, uint32_t scene, const int32_t* pos, const uint32_t* mat, uint32_t k, uint32_t* added);
/* The cursor ball (3d/sim3d.wgsl:154-176; tables per buildBallLUT,
 * 3d/app.js:212-230): centre in Q16.16, radius in world units (0, 64]. */
int sn3_set_ball(sn3_engine* e, uint32_t scene, uint32_t on, int32_t x, int32_t y, int32_t z, double radius_wu);
int sn3_fnv(sn3_engine* e, uint32_t scene, uint32_t lanes[8]);
int sn3_digest(sn3_engine* e, uint32_t scene, uint32_t acc[8]);
int sn3_chain(sn3_engine* e, uint32_t scene, uint32_t chain[8]);
int sn3_read_state(sn3_engine* e, uint32_t scene, int32_t* out, size_t words);
/* (no counterpart: the reference's 3D page has no bonds) Build-defined bonds
 * of a 3D scene, the 2D engine's bond distance constraint (src/sim.wgsl:
 * 1594-1671, the bond gather of friction :1880-1934) restated over three axes.
 * rows: n * 12 words, 6 entries per particle of {partner + 1, L0} (scene-local
 * partner index plus one, 0 ending the row; rest length in ticks >> 5, 512..5120);
 * a bond sits in both ends' rows. stiffness: Q16 in 0..65536; break_ratio: a
 * bond breaks when |d|^2 > L0^2 * break_ratio / 2^16 (0: only the hard limit).
 * Each solver iteration adds every bonded particle's correction, computed from
 * the iteration's starting positions, to its density correction; a broken
 * bond is tombstoned (bit 31 of its first word) in both rows. Replaces the
 * scene's rows; a scene load clears them; checkpoints do not carry them. */
int sn3_write_bonds(sn3_engine* e, uint32_t scene, const uint32_t* rows, size_t words, int32_t stiffness,
                    int32_t break_ratio);
int sn3_read_bonds(sn3_engine* e, uint32_t scene, uint32_t* out, size_t words);
/* Keyframe restore: n particles' state words, the substep count and the chain
 * (NULL keeps the chain). */
int sn3_write_state(sn3_engine* e, uint32_t scene, const int32_t* state, uint32_t n, uint64_t substeps,
                    const uint32_t chain[8]);
int sn3_debug_counters(sn3_engine* e, uint32_t out[16]);
int sn3_sync(sn3_engine* e);
int sn3_get_info(sn3_engine* e, uint32_t scene, sn3_info* out);
int sn3_last_timing(sn3_engine* e, float* ms, uint64_t* launches);
/* Phases: predict, sort, cellstart+gather, neighbour lists, then density and
 * solve per iteration, integrate(+hash), fold. */
int sn3_profile_substep(sn3_engine* e, uint32_t reps, float* ms, uint32_t max_phases, uint32_t* n_phases);

/* ---- device checkpoints ------------------------------------------------------
 * No counterpart in the reference (its keyframes are host copies,
 * src/demo_boot.js:104-125). A pool is one device allocation of `bytes`; a
 * checkpoint of a scene (2D: state, scratch, chain, bond rows and the
 * formation/substep clocks; 3D: state, chain and the substep clock) is copied
 * into it on the engine's stream without a host round trip and restored the
 * same way. A 2D scene's rigid bodies travel too: their rest offsets in the
 * pool, their records and drivers on the host (saving and loading such a
 * scene waits for the stream once). Loading a checkpoint into a scene rewinds (or advances) that
 * scene exactly: every later substep equals the one after the save. A 2D
 * checkpoint loads only into a scene with the same n and n_fluid. The pool
 * orders copies across engines with events, so one pool may serve several
 * engines on the same device; a pool is not thread-safe. */
typedef struct sn_ckpt_pool sn_ckpt_pool;
int sn_ckpt_pool_create(size_t bytes, int32_t device, sn_ckpt_pool** out);
void sn_ckpt_pool_destroy(sn_ckpt_pool* p);
const char* sn_ckpt_pool_last_error(const sn_ckpt_pool* p);
int sn_ckpt_pool_usage(const sn_ckpt_pool* p, size_t* used, size_t* capacity);
/* Release a checkpoint (waits for copies in flight that touch it). */
int sn_ckpt_free(sn_ckpt_pool* p, uint64_t handle);
/* Bytes a checkpoint of this scene takes now (before 256-byte rounding). */
int sn_ckpt_bytes(sn_engine* e, size_t* bytes);
/* The single-scene engine's keyframe on the device: WaterDemo.snapshot() /
 * restore() (src/demo_boot.js:286-320) without a host round trip. */
int sn_ckpt_save(sn_engine* e, sn_ckpt_pool* p, uint64_t* handle);
int sn_ckpt_load(sn_engine* e, sn_ckpt_pool* p, uint64_t handle);
int sn_batch_ckpt_bytes(sn_batch* b, uint32_t id, size_t* bytes);
int sn_batch_ckpt_save(sn_batch* b, uint32_t id, sn_ckpt_pool* p, uint64_t* handle);
int sn_batch_ckpt_load(sn_batch* b, uint32_t id, sn_ckpt_pool* p, uint64_t handle);
int sn3_ckpt_bytes(sn3_engine* e, uint32_t scene, size_t* bytes);
int sn3_ckpt_save(sn3_engine* e, uint32_t scene, sn_ckpt_pool* p, uint64_t* handle);
int sn3_ckpt_load(sn3_engine* e, uint32_t scene, sn_ckpt_pool* p, uint64_t handle);

#ifdef __cplusplus
}
#endif

#endif /* SUNA_H */
