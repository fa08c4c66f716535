/*
 * akua_pbf.h — C ABI of the GB300 Position-Based Fluids step.
 *
 * Drop-in for AkuaEngine's per-frame solver step.  Each entry point names the reference
 * interface it replaces (paths relative to the AkuaEngine source tree).  Plain pointers and sizes
 * only; every call returns a status (0 = ok, negative = error) — the reference reports no errors.
 *
 * Threading: a handle is not thread-safe.  All device work of a handle is issued on one CUDA
 * stream (the legacy default stream unless akua_pbf_set_stream is called) and is asynchronous
 * with respect to the host unless stated otherwise.
 */
#ifndef AKUA_PBF_H
#define AKUA_PBF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AKUA_PBF_ABI_VERSION 1

/* Status codes. */
#define AKUA_OK 0
#define AKUA_ERR_INVALID_ARGUMENT (-1)
#define AKUA_ERR_CUDA (-2)
#define AKUA_ERR_OUT_OF_MEMORY (-3)
#define AKUA_ERR_NOT_ATTACHED (-4)  /* step before a particle buffer was attached */
#define AKUA_ERR_DEVICE_CHECK (-5)  /* a device-side consistency check failed */
#define AKUA_ERR_TOO_LARGE (-6)     /* a size exceeds a fixed limit of the called entry point */
#define AKUA_ERR_CORRUPT (-7)       /* a state file failed its checksum */

/* Options (akua_pbf_set_options). */
#define AKUA_PBF_OPT_EXACT_MATH 0x1u /* IEEE sqrt/divide in every pair term (bit-reproducible) */
#define AKUA_PBF_OPT_RESIDENT 0x2u   /* read the attached buffer only on the first step */
#define AKUA_PBF_OPT_NO_GRAPH 0x4u   /* launch kernels one by one instead of a captured graph */

/* Solver parameters: AkuaEngine::PBFConfig, include/AkuaEngine/Simulation/PBFConfig.h:18-29. */
typedef struct akua_pbf_config {
    float restDensity;
    float particle_spacing;     /* carried; the step does not read it (as in the reference) */
    float smoothRadius;         /* kernel radius h; also the hashing cell (NeighbourSearchCUDA.cu:163) */
    float spatialHashCellSize;  /* cell used by the neighbour walk (NeighbourSearchCUDA.cu:177) */
    float relaxation;           /* epsilon in the lambda denominator */
    float vorticityEpsilon;
    float viscosity;            /* XSPH coefficient c */
    int32_t maxNeighbours;      /* list capacity per particle; table size = maxNeighbours * N */
    int32_t solverIterations;
    float gravity[3];
} akua_pbf_config;

/* Artificial pressure: AkuaEngine::LambdaCorrParams, PBFConfig.h:10-15. */
typedef struct akua_lambda_corr_params {
    int32_t enabled; /* carried; never read, as in the reference */
    float k;
    float n;
    float delta_q;
} akua_lambda_corr_params;

/* One particle record: AkuaEngine::Particle, include/AkuaEngine/Simulation/Particle.h:8-31
 * (108 bytes, 4-byte aligned).  This is also the vertex layout the reference renders from. */
typedef struct akua_particle {
    float position[3];
    float velocity[3];
    float new_position[3];
    float new_velocity[3];
    float position_delta[3];
    float vorticity[3];
    float mass;
    float density;
    float lambda;
    uint32_t hash;
    float color[4];
    float size;
} akua_particle;

typedef struct akua_pbf akua_pbf;

/* Per-handle counters (akua_pbf_get_stats). */
typedef struct akua_pbf_stats {
    int32_t numParticles;
    int32_t tableSize;
    int32_t maxNeighbours;
    int32_t solverIterations;
    int64_t steps;            /* steps issued on this handle */
    uint32_t deviceFlags;     /* bit 0: some list reached maxNeighbours; bit 1: bad table entry */
    int32_t graphCaptures;    /* how many times the step graph was (re)captured */
    uint64_t deviceBytes;     /* device memory held by the handle */
} akua_pbf_stats;

/* Debug readbacks (akua_pbf_read_debug), all for the sorted order of the last step. */
#define AKUA_DEBUG_HASHES 1           /* uint32[N]: cell hash per particle */
#define AKUA_DEBUG_ORDER 2            /* uint32[N]: pre-sort index of the particle now at slot s */
#define AKUA_DEBUG_NEIGHBOUR_COUNTS 3 /* uint32[N] */
#define AKUA_DEBUG_NEIGHBOURS 4       /* uint32[N * maxNeighbours], row i holds particle i's list */
#define AKUA_DEBUG_PARTICLES 5        /* akua_particle[N]: the solver's current state */
#define AKUA_DEBUG_LAMBDA_SUMS 6      /* float[N]: last step's accumulated lambda, record order */

/* Reference defaults of PBFConfig / LambdaCorrParams (PBFConfig.h:10-29). */
void akua_pbf_default_config(akua_pbf_config* config, akua_lambda_corr_params* corr);

/* Replaces PBFSolver::PBFSolver(int, const PBFConfig&, const LambdaCorrParams&)
 * (src/Simulation/PBFSolver.cpp:13-20).  Allocates all device memory of the handle on the
 * current device: the neighbour lists (N * maxNeighbours), the cell table (maxNeighbours * N
 * entries, PBFSolver.cpp:15) and the SoA particle state. */
int akua_pbf_create(int32_t numParticles, const akua_pbf_config* config,
                    const akua_lambda_corr_params* corr, akua_pbf** out);

/* Frees the handle and its device memory (synchronises the handle's stream first). */
int akua_pbf_destroy(akua_pbf* solver);

/* Replaces InteropResource + cudaGraphicsResourceGetMappedPointer (src/Interop/InteropResource.cpp:9-14,
 * src/CUDA/IntegrationCUDA.cu:201-204): `deviceParticles` is a device array of N particle records
 * with `strideBytes` between records (108 for akua_particle; larger strides are allowed, must be a
 * multiple of 4).  The solver reads and rewrites the records in place, leaving them sorted by cell
 * hash as the reference does.  Pass NULL to detach. */
int akua_pbf_attach_particles(akua_pbf* solver, void* deviceParticles, size_t strideBytes);

/* Replaces PBFSolver::step(const InteropResource&, float, glm::vec3, glm::vec3)
 * (src/Simulation/PBFSolver.cpp:22-78): predict, hash, sort, neighbour lists, solverIterations
 * Jacobi iterations of the density constraint, update, boundary damping, vorticity confinement and
 * XSPH viscosity over the attached buffer.  Asynchronous on the handle's stream. */
int akua_pbf_step(akua_pbf* solver, float deltaTime, const float boxMin[3], const float boxMax[3]);

/* The same step for callers that hold the particle array in host memory (stride as in
 * akua_pbf_attach_particles).  Pinned memory (cudaHostAlloc, cudaHostRegister) is read and
 * written in place by the step's import and export kernels; other memory is copied to a device
 * buffer and back.  Synchronous: returns after the records are back in `hostParticles`. */
int akua_pbf_step_host(akua_pbf* solver, void* hostParticles, size_t strideBytes, float deltaTime,
                       const float boxMin[3], const float boxMax[3]);

/* Replaces PBFSolver::setGravity(glm::vec3) (include/AkuaEngine/Simulation/PBFSolver.h:29-31). */
int akua_pbf_set_gravity(akua_pbf* solver, const float gravity[3]);

/* Boundary velocity damping coefficients; the reference hard-codes restitution 0 and friction 0.95
 * at its call site (src/Simulation/PBFSolver.cpp:64), which are the defaults here. */
int akua_pbf_set_boundary_damping(akua_pbf* solver, float restitution, float friction);

/* Cell table size; the reference fixes it to maxNeighbours * N (PBFSolver.cpp:15), the default.
 * Changing it changes every hash, hence the sorted order. */
int akua_pbf_set_table_size(akua_pbf* solver, int32_t tableSize);

/* New: PBFConfig::solverIterations after construction (the reference fixes it when the solver is
 * built, PBFSolver.cpp:13-20); 0 .. 1000. */
int akua_pbf_set_solver_iterations(akua_pbf* solver, int32_t iterations);
/* New: the CUDA stream (a cudaStream_t) all device work of this handle is issued on. */
int akua_pbf_set_stream(akua_pbf* solver, void* cudaStream);

/* New: AKUA_PBF_OPT_* flags. */
int akua_pbf_set_options(akua_pbf* solver, uint32_t options);

/* New: blocks until the handle's device work is done; reports deferred device errors. */
int akua_pbf_synchronize(akua_pbf* solver);

/* New: counters; synchronises the handle's stream. */
int akua_pbf_get_stats(akua_pbf* solver, akua_pbf_stats* stats);

/* New: copies one AKUA_DEBUG_* array to host memory (synchronous); `bytes` must match. */
int akua_pbf_read_debug(akua_pbf* solver, int32_t what, void* hostDst, size_t bytes);

/* New: how many of the library's kernels one akua_pbf_step launches with the current settings. */
int akua_pbf_kernels_per_step(akua_pbf* solver);

/* New: per-kernel timing of the next steps with CUDA events recorded on the handle's stream
 * between consecutive kernels.  While profiling, steps are launched kernel by kernel (no graph). */
typedef struct akua_kernel_time {
    char name[40];
    int32_t launches;
    double total_ms;
} akua_kernel_time;
int akua_pbf_profile_begin(akua_pbf* solver, int32_t maxSteps);
/* Ends profiling; synchronises; writes up to `capacity` entries (one per kernel name). */
int akua_pbf_profile_end(akua_pbf* solver, akua_kernel_time* out, int32_t capacity, int32_t* count);

/* No counterpart in the reference.  The step's stable radix sort of (key, value) pairs, for
 * callers that cannot allocate device memory: applications whose device memory belongs to their
 * own allocator or a fixed budget, and frame loops that cannot afford an allocation's implicit
 * device synchronisation.
 * Sorts the n pairs (keysIn[i], valsIn[i]) by the low keyBits bits of the key (higher key bits
 * are ignored), ties in input order, into keysOut / valsOut (device arrays; keysOut receives the
 * whole keys).  The inputs are not modified; no output may overlap an input or the other output
 * (AKUA_ERR_INVALID_ARGUMENT).  valsIn == NULL makes each key's index its payload.  Asynchronous
 * on cudaStream.
 * Temporary storage is one fixed device array inside the library (about 9.5 MB, held on every
 * device that loads the library until exit); nothing is allocated, and n above
 * AKUA_SORT_NOALLOC_MAX_PAIRS returns AKUA_ERR_TOO_LARGE.  The first call on a device looks up
 * that array's device address and keeps it, so make that call before any stream capture, and do
 * not call cudaDeviceReset between calls.  Every call shares the array: calls that overlap on the
 * GPU race and must be ordered by the caller. */
#define AKUA_SORT_NOALLOC_MAX_PAIRS (1 << 20)
int akua_sort_pairs_noalloc(const uint32_t* keysIn, const uint32_t* valsIn, uint32_t* keysOut,
                            uint32_t* valsOut, int32_t n, int32_t keyBits, void* cudaStream);

/* ---- Batches of independent scenes.  No counterpart in the reference (one solver per scene). ---
 * One handle steps many scenes at once: their particle records lie one after another in the
 * attached array (scene k at records [first_k, first_k + numParticles_k)), every kernel of a step
 * covers all of them, and each scene's result is bit-identical to stepping it alone with its own
 * solver (same hash table size maxNeighbours * N_k, box and gravity): the hash keys of scene k
 * are offset by maxNeighbours * first_k, so one sort orders the batch by (scene, hash) and each
 * scene's records come back sorted within its own range.  A batch handle takes
 * akua_pbf_step_batch / akua_pbf_set_scene in place of akua_pbf_step / akua_pbf_step_host /
 * akua_pbf_set_gravity / akua_pbf_set_table_size (those return AKUA_ERR_INVALID_ARGUMENT). */
typedef struct akua_scene_desc {
    int32_t numParticles;
    float gravity[3];
    float boxMin[3];
    float boxMax[3];
} akua_scene_desc;
/* At most 65535 scenes; shared PBFConfig / LambdaCorrParams. */
int akua_pbf_create_batch(int32_t numScenes, const akua_scene_desc* scenes,
                          const akua_pbf_config* config, const akua_lambda_corr_params* corr,
                          akua_pbf** out);
/* One step of every scene of the batch over the attached records; asynchronous. */
int akua_pbf_step_batch(akua_pbf* solver, float deltaTime);
/* Changes scene `scene`'s gravity and box (numParticles must stay the same). */
int akua_pbf_set_scene(akua_pbf* solver, int32_t scene, const akua_scene_desc* desc);

/* ---- Launch shapes.  No counterpart in the reference (fixed 256-thread blocks). ---------------
 * The neighbour-pair kernels (in this order: density and lambda, delta with correction, last
 * delta with update and damping, vorticity, confinement, XSPH) run with a block size chosen per
 * kernel from 64, 128 and 256 threads; results do not depend on it. */
#define AKUA_PBF_PAIR_KERNELS 6
int akua_pbf_set_pair_blocks(akua_pbf* solver, const int32_t blocks[AKUA_PBF_PAIR_KERNELS]);
int akua_pbf_get_pair_blocks(akua_pbf* solver, int32_t blocks[AKUA_PBF_PAIR_KERNELS]);
/* The neighbour walk's tile shape: its block size (64, 128 or 256 threads) and how many list
 * entries per particle it stages in shared memory before writing them out (16, 32, or 48 with 64
 * or 128 threads); lists do not depend on it.  Default 128 / 32. */
int akua_pbf_set_search_shape(akua_pbf* solver, int32_t block, int32_t staged);
int akua_pbf_get_search_shape(akua_pbf* solver, int32_t* block, int32_t* staged);
/* Autotuner: times every candidate block size of every pair kernel, then every walk tile shape,
 * over `steps` profiled steps (after one warm-up step) started from a copy of the attached
 * records, and keeps the fastest per kernel (the pair kernels' written to blocksOut when not
 * NULL; the walk's shape read back with akua_pbf_get_search_shape).  The attached records, the
 * step count, pending captures and the lambda sums are left as they were.  boxMin/boxMax as for
 * akua_pbf_step (NULL for a batch, whose scenes carry their boxes).  Synchronous. */
int akua_pbf_autotune(akua_pbf* solver, float deltaTime, const float boxMin[3],
                      const float boxMax[3], int32_t steps, int32_t* blocksOut);

/* ---- SDF obstacles.  The reference clamps particles to the box and plans a proper boundary in its
 * place (ConstraintSolverCUDA.cu:131-134); here solid shapes given by signed distance functions
 * are added to the box: after each Jacobi correction (and the box clamp) a particle within
 * minDist of an obstacle moves by stiffness * (minDist - phi) along the SDF gradient (the box
 * clamp's rule, 0.025 and 0.5 there), and the update damps the velocity against each obstacle as
 * against the box's planes.  No shapes (the default): the reference's step exactly. */
#define AKUA_SDF_SPHERE 1   /* a = centre, radius */
#define AKUA_SDF_BOX 2      /* a = centre, b = half extents, radius = corner rounding */
#define AKUA_SDF_CAPSULE 3  /* segment a-b, radius */
#define AKUA_SDF_PLANE 4    /* a = unit normal into the fluid, b[0] = offset: solid where a.x < b[0] */
#define AKUA_SDF_MAX_SHAPES 64
typedef struct akua_sdf_shape {
    int32_t type;
    float a[3];
    float b[3];
    float radius;
} akua_sdf_shape;
int akua_pbf_set_sdf_shapes(akua_pbf* solver, const akua_sdf_shape* shapes, int32_t count,
                            float minDist, float stiffness);

/* ---- State files.  No counterpart in the reference (its scene is rebuilt in code each run). ----
 * A file holds the particle records of a simulation and what resuming it needs: the solver
 * parameters, box, time step, step count and table size, optionally the per-particle lambda sums
 * (warm start) and the scenes of a batch.  Records plus parameters determine every later step, so
 * a run resumed from a file continues bit for bit.  Layout: a 256-byte header, the records, the
 * lambda sums (float[N]) if sections & AKUA_STATE_LAMBDA_SUMS, the scene descriptors if
 * numScenes > 0; crc32 (IEEE, as zlib's) covers everything after the header. */
#define AKUA_STATE_VERSION 1
#define AKUA_STATE_HEADER_BYTES 256
#define AKUA_STATE_LAMBDA_SUMS 0x1u
typedef struct akua_state_header {
    char magic[8];                /* "AKUAPBF\0" */
    uint32_t version;             /* AKUA_STATE_VERSION */
    uint32_t recordBytes;         /* 108 */
    int64_t numParticles;
    int64_t step;                 /* steps simulated before this state */
    akua_pbf_config config;
    akua_lambda_corr_params corr;
    float boxMin[3];
    float boxMax[3];
    float deltaTime;
    uint32_t tableSize;
    uint32_t sections;            /* AKUA_STATE_* bits */
    int32_t numScenes;            /* 0: one scene */
    uint32_t crc32;               /* written by akua_state_save */
    uint32_t options;             /* AKUA_PBF_OPT_* of the run */
    uint8_t reserved[112];
} akua_state_header;
/* Zeroes `header` and fills magic, version and recordBytes. */
void akua_state_init_header(akua_state_header* header);
/* Writes a state file; lambdaSums must be given exactly when the header's sections say so, and
 * scenes exactly when numScenes > 0.  Host memory only. */
int akua_state_save(const char* path, const akua_state_header* header, const void* records,
                    const float* lambdaSums, const akua_scene_desc* scenes);
int akua_state_read_header(const char* path, akua_state_header* header);
/* Reads a state file into host memory (records: capacity records; lambdaSums may be NULL to skip
 * them; scenes: sceneCapacity descriptors); AKUA_ERR_CORRUPT when the checksum does not match. */
int akua_state_load(const char* path, akua_state_header* header, void* records, int64_t capacity,
                    float* lambdaSums, akua_scene_desc* scenes, int32_t sceneCapacity);
/* Sets the per-particle lambda sums the next step reads as "the previous step's" (record order;
 * the counterpart of AKUA_DEBUG_LAMBDA_SUMS, for resuming a warm-started run). */
int akua_pbf_set_lambda_sums(akua_pbf* solver, const float* hostSums, int64_t count);

/* ---- Headless point-splat renderer.  Replaces the reference's GL particle pass
 * (assets/shaders/fluidParticle.vert/.frag, src/Rendering/Renderer.cpp:29-50) with CUDA kernels
 * writing an RGBA8 image: points of size Particle::size / distance, a round splat with
 * colour * exp(-3 r^2) (r = distance from the splat centre in units of its size), depth test
 * LESS, no blending, clear colour (0.15, 0.15, 0.18, 1). */
typedef struct akua_camera {
    float position[3];
    float gaze[3];      /* view direction */
    float up[3];        /* world up */
    float fovDegrees;   /* vertical field of view */
    float nearZ;
    float farZ;
} akua_camera;
/* The reference's camera at start-up (CameraConfig.h:8-16, Application.cpp:17-18). */
void akua_camera_default(akua_camera* camera);
/* Column-major view (lookAt(position, position + gaze, up)), projection (perspective, depth in
 * [-1, 1]) and projection * view; any output may be NULL. */
int akua_camera_matrices(const akua_camera* camera, float aspect, float* view, float* projection,
                         float* viewProjection);
typedef struct akua_splat akua_splat;
int akua_splat_create(int32_t width, int32_t height, akua_splat** out);
int akua_splat_destroy(akua_splat* renderer);
/* Renders n particle records (device memory, strideBytes apart) into deviceRGBA (width * height
 * pixels, R in the low byte, row 0 at the top); asynchronous on cudaStream. */
int akua_splat_render(akua_splat* renderer, const void* deviceParticles, size_t strideBytes,
                      int32_t n, const akua_camera* camera, uint32_t* deviceRGBA,
                      void* cudaStream);

/* ---- Learned lambda warm start.  No counterpart in the reference. ----------------------------
 * A network of 8 inputs, three hidden layers of 64 SiLU units and one output, BF16 weights and
 * activations on the tensor cores with FP32 accumulation, trained on the GPU.  It predicts, from
 * per-particle features at the start of a step, the lambda a 20-iteration solve accumulates over
 * the step; with a network attached, a step's first Jacobi iteration uses that prediction instead
 * of the one-step estimate and the remaining iterations run unchanged.
 * Features (float[8] per particle): rho/rho0 - 1, neighbours / 32, the lambda denominator without
 * epsilon, iteration 1's lambda, the previous step's accumulated lambda, the mean rho_j/rho0 - 1
 * of the neighbours, the SPH divergence of the predicted velocity, |predicted velocity|.
 * Parameters (float[AKUA_MLP_PARAMS], FP32 master copy): W1[64][8], b1[64], W2[64][64], b2[64],
 * W3[64][64], b3[64], w4[64], b4.  Normalisation (float[AKUA_MLP_NORM]): mean[8], inv_std[8] of
 * the features, the output scale (the network's output times it is the estimate p of the
 * accumulated lambda) and the blend b: the lambda used (by a step, and by akua_mlp_forward) is
 * lambda0 + b (p - lambda0) with lambda0 = feature 3 (b = 1 gives p; b = 0 the plain solver's
 * lambda).  In a warm-started step, p itself is what the next step sees as the previous step's
 * accumulated lambda. */
#define AKUA_MLP_INPUTS 8
#define AKUA_MLP_HIDDEN 64
#define AKUA_MLP_PARAMS 8961
#define AKUA_MLP_NORM 18
typedef struct akua_mlp akua_mlp;
/* Allocates the network on the current device (zero parameters, identity normalisation). */
int akua_mlp_create(akua_mlp** out);
int akua_mlp_destroy(akua_mlp* net);
/* Host copies of the FP32 parameters; setting them resets the optimiser state.  Synchronous. */
int akua_mlp_set_params(akua_mlp* net, const float* hostParams, int32_t count);
int akua_mlp_get_params(akua_mlp* net, float* hostParams, int32_t count);
int akua_mlp_set_normalization(akua_mlp* net, const float* hostNorm, int32_t count);
/* out[i] = network(features[8 i .. 8 i + 7]) for n particles (device arrays); asynchronous. */
int akua_mlp_forward(akua_mlp* net, const float* deviceFeatures, float* deviceOut, int32_t n,
                     void* cudaStream);
/* Gradient of L = (1/n) sum_i (out_i - target_i)^2 / outScale^2 with respect to the FP32
 * parameters (hostGrad[AKUA_MLP_PARAMS], may be NULL) and L itself (hostLoss, may be NULL);
 * synchronous.  Returns AKUA_ERR_DEVICE_CHECK if a tensor-core wait timed out. */
int akua_mlp_gradient(akua_mlp* net, const float* deviceFeatures, const float* deviceTargets,
                      int32_t n, float* hostGrad, float* hostLoss, void* cudaStream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on L over the n given samples; asynchronous. */
int akua_mlp_adam_step(akua_mlp* net, const float* deviceFeatures, const float* deviceTargets,
                       int32_t n, float learningRate, void* cudaStream);
/* Waits for the stream; AKUA_ERR_DEVICE_CHECK if any kernel of the network reported a timeout. */
int akua_mlp_synchronize(akua_mlp* net, void* cudaStream);
/* Attaches a network (NULL detaches: the plain solver) to a solver on the same device.  Needs
 * solverIterations >= 1.  The network must outlive the attachment. */
int akua_pbf_set_warm_start(akua_pbf* solver, akua_mlp* net);
/* Makes the next step write, in one consistent particle order, the features of every particle at
 * its start (deviceFeatures, float[8 N]) and the lambda its iterations accumulated
 * (deviceTargets, float[N]): training pairs when the step runs a long plain solve.  NULLs cancel.
 * Needs solverIterations >= 1. */
int akua_pbf_capture_training(akua_pbf* solver, float* deviceFeatures, float* deviceTargets);
/* Keeps the per-particle lambda sum of every step (and the features) even without a capture or a
 * network, so that the "previous step's accumulated lambda" feature is valid at any step; a
 * capture turns it on.  Needs solverIterations >= 1. */
int akua_pbf_set_lambda_tracking(akua_pbf* solver, int32_t enabled);
/* Density-constraint error of the last step: C_i = rho_i / rho0 - 1 at the positions the step
 * ended with, over that step's neighbour lists; *maxError = max_i max(C_i, 0),
 * *meanAbsError = mean_i |C_i|.  Synchronous. */
int akua_pbf_density_error(akua_pbf* solver, float* maxError, float* meanAbsError);

const char* akua_pbf_status_string(int status);
int akua_pbf_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* AKUA_PBF_H */
