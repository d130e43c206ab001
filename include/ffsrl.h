/*
 * ffsrl.h -- C ABI of libffsrl_cuda.so, the GB300 (sm_103a) implementation of FF-SRL's
 * multi-environment soft-tissue step, BVH refit and ray-cast renderer.
 *
 * Every entry point takes plain pointers and sizes.  Device arrays are owned by the
 * caller (the Python layer hands it torch tensors' data_ptr()).  Streams are passed as
 * `void*` holding a cudaStream_t (NULL = legacy default stream).  Calls return an
 * ffsrl_status; ffsrl_last_error() gives a message for the calling thread's last error.
 *
 * Array layouts follow the reference's SimModelDO (FF_SRL/FF_SRL/modelDO.py:1141-1246):
 * every array is the concatenation over environments, vec3 arrays are float32 AoS
 * (x,y,z per element), index arrays are int32 holding GLOBAL indices.
 */
#ifndef FFSRL_H
#define FFSRL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFSRL_ABI_VERSION 2

typedef enum {
    FFSRL_OK = 0,
    FFSRL_ERR_INVALID_ARGUMENT = 1,
    FFSRL_ERR_CUDA = 2,
    FFSRL_ERR_OUT_OF_MEMORY = 3,
    FFSRL_ERR_BUDGET = 4,          /* serving: admission would exceed the HBM budget */
    FFSRL_ERR_TIMEOUT = 5,         /* a bounded wait gave up */
    FFSRL_ERR_UNSUPPORTED = 6,
    FFSRL_ERR_NONFINITE = 7,       /* NaN/Inf detected in an environment's state */
    FFSRL_ERR_STACK_OVERFLOW = 8,  /* BVH traversal stack exhausted */
    FFSRL_ERR_BUSY = 9,            /* serving: no free slot */
    FFSRL_ERR_NOT_FOUND = 10
} ffsrl_status;

/* ---- constraint selection (ffsrl_params.flags) --------------------------------- */
#define FFSRL_VOLUME         (1u << 0) /* volumeConstraints      integrator.py:444-504 */
#define FFSRL_DISTANCE       (1u << 1) /* distanceConstraints    integrator.py:65-109  */
#define FFSRL_NEOHOOKEAN     (1u << 2) /* neoHookeanConstraints  integrator.py:578-698 */
#define FFSRL_DISTANCE_XPBD  (1u << 3) /* distanceConstraintsXPBD integrator.py:191-240 */
#define FFSRL_VOLUME_XPBD    (1u << 4) /* volumeConstraintsXPBD  integrator.py:507-576 */
#define FFSRL_DRAG           (1u << 5) /* dragConstraintsDO      integrator.py:412-442 */
#define FFSRL_CONNECTORS     (1u << 6) /* triToPointDistanceConstraintsDO integrator.py:300-353 */
#define FFSRL_COLLIDE        (1u << 7) /* collideLaparoscopeDO   integrator.py:981-1050 */
/* the launch sequence of SimIntegratorDO.stepModel (integrator.py:1640-1741) */
#define FFSRL_REFERENCE_STEP (FFSRL_VOLUME | FFSRL_DISTANCE | FFSRL_DRAG | FFSRL_CONNECTORS | FFSRL_COLLIDE)

/* ---- model: the arrays of SimModelDO (modelDO.py:1141-1246) -------------------- */
typedef struct {
    int32_t num_vertices, num_tetrahedrons, num_edges, num_triangles, num_connectors, num_envs;

    float* vertex;              /* [3V] */
    float* predicted_vertex;    /* [3V] */
    float* velocity;            /* [3V] */
    float* dp;                  /* [3V] correction accumulator (reference: SimModelDO.dP) */
    int32_t* constraints_number;/* [V]  (reference: SimModelDO.constraintsNumber) */
    float* collision_dp;        /* [3V] collision response accumulator (see collide) */
    const float* inverse_mass;  /* [V] */

    const int32_t* tetrahedron;            /* [4T] */
    const float* tetrahedron_rest_volume;  /* [T]  |V0| */
    const float* active_tetrahedron;       /* [T] */
    const float* tetrahedron_dm_inv;       /* [9T] row-major Dm^-1 (Neo-Hookean) */
    float* tetrahedron_lambda;             /* [T]  XPBD volume multipliers */
    const float* xpbd_rest_volume;         /* [T]  signed rest volume (XPBD volume) */

    const int32_t* edge;                   /* [2E] */
    const float* edge_rest_length;         /* [E] */
    const float* active_edge;              /* [E] */
    float* edge_lambda;                    /* [E]  XPBD distance multipliers */

    const int32_t* triangle;               /* [3F] surface triangles (vertex ids) */
    const int32_t* tri_to_env;             /* [F] */
    const int32_t* hole;                   /* [F] */
    const int32_t* vertex_to_env;          /* [V] */
    const float* active_drag_constraint;   /* [V] */

    /* instrument, 4 entries per env: 0..2 capsules (rod, left clamp, right clamp),
       3 = drag point (modelDO.py:218-245) */
    const float* laparoscope_base;         /* [3*4N] */
    const float* laparoscope_tip;          /* [3*4N] */
    const float* laparoscope_radius;       /* [4N] */
    int32_t* laparoscope_in_collision;     /* [N] */

    const int32_t* connector_triangle_id;  /* [3C] */
    const float* connector_tri_bar;        /* [3C] */
    const int32_t* connector_vertex_id;    /* [C] */
    const float* connector_rest_dist;      /* [C] */

    /* per-env ranges, [N+1] prefix arrays (optional for the reference-shaped step) */
    const int32_t* env_vertex_start;
    const int32_t* env_tet_start;
    const int32_t* env_edge_start;
    const int32_t* env_tri_start;
} ffsrl_model;

/* ---- solver parameters (SimModelDO.__init__ kwargs, modelDO.py:774-802) -------- */
typedef struct {
    int32_t substeps;            /* simSubsteps */
    int32_t iterations;          /* simConstraints */
    uint32_t flags;              /* FFSRL_* selection */
    float dt;                    /* simDt = 1/fps/substeps, as float32 */
    float gravity[3];
    float velocity_dampening;
    float ground_level;
    float ks_distance, ks_volume, ks_contact, ks_drag;
    float volume_compliance, deviatoric_compliance;   /* Neo-Hookean (1/lambda, 1/mu) */
    float distance_compliance, volume_compliance_xpbd;/* XPBD alpha; alpha/dt^2 is formed in double */
    float connector_mass_weight_ratio, connector_ks, connector_rest_length_mul;
} ffsrl_params;

/* ---- BVH (bvh.py:144-518), per-env AABBs over shared or per-env topologies ------ */
typedef struct {
    int32_t num_envs;
    int32_t num_topologies;
    const int32_t* env_topology;     /* [N] topology used by env e */
    const int32_t* env_node_offset;  /* [N] first AABB slot of env e */
    const int32_t* env_face_offset;  /* [N] global vis-face id of env e's local face 0 */
    const int32_t* topo_node_offset; /* [M+1] node range of each topology */
    const int32_t* topo_tri_offset;  /* [M+1] tri-map range of each topology */
    const int32_t* topo_max_level;   /* [M] */
    const int32_t* left_node;        /* [nodes] -1 = leaf; children leftNode, leftNode+1 (topology-local) */
    const int32_t* first_tri_id;     /* [nodes] into the topology's tri map */
    const int32_t* tri_count;        /* [nodes] */
    const int32_t* level;            /* [nodes] */
    const int32_t* tri_id;           /* [tris] local face ids (triMap) */
    float* aabb_min;                 /* [3 * total_env_nodes] */
    float* aabb_max;                 /* [3 * total_env_nodes] */
    int32_t total_env_nodes;
    int32_t total_topology_nodes;
    int32_t max_level;               /* max over topologies */
    /* optional, for the fused refit: each topology's node ids grouped by level, deepest
       level first; group g of topology m is level_node[level_start[topo_level_offset[m] + g]
       .. level_start[topo_level_offset[m] + g + 1]) holding level topo_max_level[m] - g */
    const int32_t* level_node;       /* [total_topology_nodes] topology-local node ids */
    const int32_t* level_start;      /* [sum_m (topo_max_level[m] + 2)] absolute offsets */
    const int32_t* topo_level_offset;/* [M+1] */
    /* optional traversal copies written by the refit (both or neither):
       node_box[2n] = (min.xyz, leftNode), node_box[2n+1] = (max.xyz, first*256 + min(count,255))
       per env node; tri_pos[12k..12k+8] = the three vertices of the k-th triangle in
       tri-map order (k = env_face_offset[e] + position in the env's topology map),
       12k+9..12k+11 padding, so each triangle is three 16-byte loads; 16-byte aligned */
    float* node_box;                 /* [8 * total_env_nodes] */
    float* tri_pos;                  /* [12 * total env faces] */
    /* optional [total env faces]: the global face whose vertices enter a leaf's box in
       place of face f (NULL: f itself).  Reproduces the reference refit's face shift at
       the object boundaries (bvh.py:66-74 uses `>` where render.py:462-470 uses `>=`);
       the traversal and tri_pos always use f.  Every entry must be a valid face id. */
    const int32_t* refit_source;
} ffsrl_bvh;

/* ---- ray-cast renderer (render.py:826-1196) ------------------------------------ */
typedef struct {
    int32_t num_envs;
    int32_t resolution;              /* R: output is R x R per env */
    int32_t num_vis_points;
    int32_t num_vis_faces;
    const float* vis_point;          /* [3P] allVisPoint */
    const int32_t* vis_face;         /* [3Fv] global point ids */
    const float* vis_point_color;    /* [3P] */
    float* normal_sum;               /* [3P] scratch */
    float* vertex_normal;            /* [3P] */
    const int32_t* point_face_start; /* [P+1] point -> incident faces, ascending face id */
    const int32_t* point_face;
    int32_t num_cameras;             /* 1 (shared, as the reference) or num_envs */
    const float* camera_pos;         /* [3C] */
    const float* camera_rot;         /* [4C] quaternion x,y,z,w */
    float camera_tan;                /* vertical_aperture / (2 * 50) */
    float camera_aspect;
    int32_t num_lights;
    const float* light_dir;          /* [3L] */
    const float* light_intensity;    /* [L] */
    float* color;                    /* [N*R*R*3] vertex-colour Lambert (mode 3) */
    float* depth;                    /* [N*R*R]   t/50 (mode 4, one channel) */
    float* rays;                     /* [N*(2R)^2*3] per-ray scratch, reference-shaped path only */
    float* ray_depth;                /* [N*(2R)^2]   per-ray scratch, reference-shaped path only */
    int32_t* error_flag;             /* [1] set to FFSRL_ERR_STACK_OVERFLOW by an overflowing ray */
    const int32_t* env_point_start;  /* [N+1] each env's visual-point range (for the *_envs calls) */
    /* shading of `color` (drawSimBVHKernelManyEnvs, render.py:350-409): 0 grayscale, 1 texture
       (vertex colour for envs without one), 2 normal map (no lighting), 3 vertex colour,
       4 depth map (t/50 in all three channels); 0, 1 and 3 are Lambert-lit.  `depth` is t/50
       in every mode.  Values outside 0..4 are rejected. */
    int32_t render_mode;
    /* textures (texture mode; NULL env_objects: no textures).  An env's visual faces are
       its objects' faces one after another (soft mesh, rigid meshes, instrument); each
       object may have a texture (modelDO.py:1052-1127).  texel (x, y) of a texture is
       first + y + x*S (render.py:139-142). */
    const float* texture;            /* [3 * texels] RGB in [0, 1], every texture one after another */
    const int32_t* env_objects;      /* [2N] per env: first entry in object_texture, number of objects */
    const int32_t* object_texture;   /* [5 per object]: first env-local face, first texel, side S
                                        (0 = no texture: vertex colour), first tex coord, first tex index */
    const float* tex_coords;         /* [2T] (u, v) */
    const int32_t* tex_indices;      /* 3 per object-local face: tex coords relative to the object's first */
} ffsrl_render;

/* ---- library ---------------------------------------------------------------- */
int32_t ffsrl_abi_version(void);
const char* ffsrl_last_error(void);
/* bytes of dynamic shared memory the device allows per block (0 without a GPU) */
int32_t ffsrl_device_info(int32_t* sm_count, int32_t* max_smem_per_block, int32_t* cc_major, int32_t* cc_minor);

/* One SimIntegratorDO.stepModel (integrator.py:1640-1741): substeps x (gravity,
   iterations x (constraints, applyConstraints, drag, connectors, collide), bounds,
   PBDStep), one kernel launch per reference kernel, float atomics as the reference. */
int32_t ffsrl_step_model(const ffsrl_model* model, const ffsrl_params* params, void* stream);

/* No counterpart in the reference.  ffsrl_step_model for callers that cannot allocate
   device memory (for example a host application that has reserved the device's memory
   for its own pool, or a control loop that must never wait on the allocator): the
   correction, count and contact accumulators come from one array compiled into the
   library instead of model->dp / constraints_number / collision_dp, which are ignored.
   At most 65536 vertices (larger models are rejected with FFSRL_ERR_INVALID_ARGUMENT);
   the array is cleared at the start of every call and shared by all calls, so calls
   that overlap on the GPU race; connector corrections do not carry over between calls.
   The first call on a device looks up the array's address; make it before any stream
   capture. */
int32_t ffsrl_step_model_noalloc(const ffsrl_model* model, const ffsrl_params* params, void* stream);

/* remapAToBKernel (utils.py:32-42): dst[map[2i]] = src[map[2i+1]] for i < count */
int32_t ffsrl_remap(float* dst, const float* src, const int32_t* map, int32_t count, void* stream);

/* remapAToBKernel for the listed envs only: the pairs of env e are map[2*point_start[e]
   .. 2*point_start[e+1]) (device arrays; point_start is the prefix of each env's pair
   count, its soft-mesh visual points -- rigid and instrument points have no pair). */
int32_t ffsrl_remap_envs(float* dst, const float* src, const int32_t* map, const int32_t* point_start,
                         const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream);

/* updateClampsDragKernel (modelDO.py:247-279): for every vertex of an env whose drag
   update flag is set, drag = (state==1 && |x - tip[4e+3]| < radius) ? 1 : 0 */
int32_t ffsrl_update_clamps_drag(const float* positions, const int32_t* vertex_to_env, const float* laparoscope_tip,
                                 float* drag, float lookup_radius, const int32_t* state, const int32_t* update,
                                 int32_t num_vertices, void* stream);
/* forceClampsDragKernel (modelDO.py:281-289): drag[env_id[i]*verts_per_env + vertex_id] = on */
int32_t ffsrl_force_clamps_drag(float* drag, int32_t vertex_id, const int32_t* env_id, int32_t num, float on,
                                int32_t verts_per_env, void* stream);
/* Grasp the nearest vertex of each env's candidate list (surface vertices) within
   `radius` of tip[4e+3]: drag=1 for it when clamp[e] != 0, every candidate of the env
   set to 0 when clamp[e] == 0.  cand_start is an [N+1] prefix array. */
int32_t ffsrl_grasp_nearest(const float* positions, const int32_t* cand_start, const int32_t* cand,
                            const float* laparoscope_tip, const int32_t* clamp, float radius, float* drag,
                            int32_t num_envs, void* stream);
/* ffsrl_grasp_nearest for the listed envs only: clamp[i] applies to env env_ids[i]
   (device arrays); ids outside [0, num_envs) are skipped. */
int32_t ffsrl_grasp_nearest_envs(const float* positions, const int32_t* cand_start, const int32_t* cand,
                                 const float* laparoscope_tip, const int32_t* clamp, float radius, float* drag,
                                 const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream);
/* Translate env env_ids[i]'s instrument by disp[3i..3i+2] (device arrays); ids outside
   [0, num_envs) are skipped. */
int32_t ffsrl_move_tool_envs(float* laparoscope_base, float* laparoscope_tip, const float* disp,
                             const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream);
/* Return the listed envs to their rest state (resetFixedModel, modelDO.py:1589-1622, for
   an env list): vertex = initial_vertex and velocity = 0 over each env's vertex range
   [env_vertex_start[e], env_vertex_start[e+1]), grasp flags 0, instrument base/tip =
   their initial values, contact count 0, and -- when xform is not NULL -- the 7 instrument
   transforms (112 floats per env) their initial values.  Device arrays; ids outside
   [0, num_envs) are skipped.  One launch for any number of envs. */
int32_t ffsrl_reset_envs(float* vertex, float* velocity, float* active_drag, const float* initial_vertex,
                         float* laparoscope_base, float* laparoscope_tip, const float* initial_base,
                         const float* initial_tip, int32_t* in_collision, float* xform, const float* initial_xform,
                         const int32_t* env_vertex_start, const int32_t* env_ids, int32_t n, int32_t num_envs,
                         void* stream);
/* ---- instrument kinematics (modelDO.py:26-416, 1331-1419, 1552-1587) -------------
   xform: 7 transforms per env, [112 * num_envs] floats, each a row-major 4x4 holding the
   transpose of the column-vector transform, as the reference stores them (slots: 0 rod
   capsule, 1 left clamp, 2 right clamp, 3 rotation centre, 4 and 5 clamp pivots, 6 rod).
   height: [4 * num_envs] capsule heights (rod, left clamp, right clamp, unused).  Every
   call ends by writing the 4 capsule ends per env into base/tip [4 * num_envs * 3]
   (updateLaparoscopeKernel, modelDO.py:222-245); entry 3's tip is the drag point.
   All arrays are device arrays unless stated. */
int32_t ffsrl_instrument_update(float* xform, float* base, float* tip, const float* height, int32_t num_envs,
                                void* stream);
/* applyActions (modelDO.py:1331-1362, applyActionsKernel :161-190): actions [5 * num_envs]
   = rod forward, rod roll, rotation-centre x, rotation-centre y, clamp opening (rad);
   drag_cut_heat / drag_cut_heat_update [3 * num_envs] carry the clamp's grasp state. */
int32_t ffsrl_instrument_apply_actions(float* xform, const float* actions, int32_t* drag_cut_heat,
                                       int32_t* drag_cut_heat_update, float* base, float* tip, const float* height,
                                       int32_t num_envs, void* stream);
/* applyCartesianActions[InWorkspace] (modelDO.py:1364-1404): actions [3 * num_envs] move
   each effector; workspace = HOST array {low x, y, z, high x, y, z} or NULL for none;
   violation [num_envs] (may be NULL) flags envs whose action was clipped. */
int32_t ffsrl_instrument_cartesian(float* xform, const float* actions, const float* workspace, int32_t* violation,
                                   float* base, float* tip, const float* height, int32_t num_envs, void* stream);
/* ffsrl_instrument_cartesian for the listed envs: actions[3i..3i+2] move env env_ids[i];
   ids outside [0, num_envs) are skipped. */
int32_t ffsrl_instrument_cartesian_envs(float* xform, const float* actions, const float* workspace, int32_t* violation,
                                        float* base, float* tip, const float* height, const int32_t* env_ids,
                                        int32_t n, int32_t num_envs, void* stream);
/* setRotationCenter (modelDO.py:1570-1587): the rotation centre takes the pose
   T(translation) Rx Ry Rz(rotation), [3 * num_envs] each, carrying the instrument. */
int32_t ffsrl_instrument_set_rotation_center(float* xform, const float* translation, const float* rotation,
                                             float* base, float* tip, const float* height, int32_t num_envs,
                                             void* stream);
/* transformSimLaparoscopeMeshData (modelDO.py:1446-1473, updateLaparoscopeMeshKernel
   modelDO.py:202-216): the instrument's visual points of each env,
   vis_point[env_first_point[e] + i] = transform point_slot[i] of env e applied to
   local_point[i], i < num_points.  One local shape [3 * num_points] serves every env (the
   reference keeps a copy per env); slots outside 0..6 are skipped.  env_ids NULL: all envs
   (n must equal num_envs); otherwise the n listed envs. */
int32_t ffsrl_instrument_visual_update(const float* xform, const float* local_point, const int32_t* point_slot,
                                       int32_t num_points, float* vis_point, const int32_t* env_first_point,
                                       const int32_t* env_ids, int32_t n, int32_t num_envs, void* stream);
/* Rigidly translate each env's instrument (4 bases + 4 tips) by disp[3e..3e+2]. */
int32_t ffsrl_move_tool(float* laparoscope_base, float* laparoscope_tip, const float* disp, int32_t num_envs,
                        void* stream);

/* ---- BVH ---------------------------------------------------------------------- */
/* Host build for one mesh: binned SAH (bvh.py:281-518).  Output capacity 2*F nodes;
   returns the node count in *num_nodes and the deepest level in *max_level.
   aabb_min/max receive the build-time float bounds. */
int32_t ffsrl_bvh_build_host(const float* points, const int32_t* faces, int32_t num_points, int32_t num_faces,
                             int32_t bins, int32_t* left_node, int32_t* first_tri_id, int32_t* tri_count,
                             int32_t* level, int32_t* tri_id, float* aabb_min, float* aabb_max,
                             int32_t* num_nodes, int32_t* max_level);
/* refitBVHLoop (bvh.py:419-440): one launch of refitBVHLevel per level, deepest first. */
int32_t ffsrl_bvh_refit_levels(const ffsrl_bvh* bvh, const float* vis_point, const int32_t* vis_face, void* stream);
/* Same result in one launch: one block per env walks its tree bottom-up. */
int32_t ffsrl_bvh_refit_fused(const ffsrl_bvh* bvh, const float* vis_point, const int32_t* vis_face, void* stream);

/* ffsrl_bvh_refit_fused for the listed envs only (device array of env ids). */
int32_t ffsrl_bvh_refit_fused_envs(const ffsrl_bvh* bvh, const float* vis_point, const int32_t* vis_face,
                                   const int32_t* env_ids, int32_t n, void* stream);

/* ---- renderer ------------------------------------------------------------------- */
/* renderFunctionNew (render.py:975-1022): zero, vertex_normal_sum (atomics), normalize,
   drawSimBVHKernelManyEnvs over (2R)^2 rays per env, downsample_kernel. */
int32_t ffsrl_render_reference(const ffsrl_render* r, const ffsrl_bvh* bvh, void* stream);
/* Same images: normals by CSR gather in face order, one thread per ray with a register
   stack, the 2x2 downsample fused through warp shuffles. */
int32_t ffsrl_render_fused(const ffsrl_render* r, const ffsrl_bvh* bvh, void* stream);

/* ffsrl_render_fused for the listed envs only (device array of env ids): their vertex
   normals (needs r->env_point_start) and images; other envs are not touched. */
int32_t ffsrl_render_fused_envs(const ffsrl_render* r, const ffsrl_bvh* bvh, const int32_t* env_ids, int32_t n,
                                void* stream);

/* ---- batched step ------------------------------------------------------------------ */
typedef struct ffsrl_batch ffsrl_batch;
/* Arithmetic of the batched step's constraint projections.  REFERENCE: each constraint
   is evaluated with the reference kernel's expressions and association order, IEEE
   division and square root, no fused multiply-add (per-constraint corrections equal the
   serial restatement's).  FAST: one hardware reciprocal or reciprocal square root per
   constraint, the Neo-Hookean constraint through M = Dm^-1 Dm^-T, multiply-add
   contraction. */
#define FFSRL_ARITH_REFERENCE 0
#define FFSRL_ARITH_FAST      1
/* Accumulation of per-vertex corrections.  FIXED: 32-bit fixed point per env scale with
   an exact 64-bit side path (deterministic; the same bits alone or in any batch).
   KAHAN: float32 (sum, compensation) pairs, compensated summation.  ATOMIC: plain
   float32 atomics, as the reference accumulates. */
#define FFSRL_ACC_FIXED  0
#define FFSRL_ACC_KAHAN  1
#define FFSRL_ACC_ATOMIC 2
typedef struct {
    int32_t block_threads;   /* 0 = default per size class */
    int32_t arithmetic;      /* FFSRL_ARITH_* (0 = reference) */
    int32_t accumulation;    /* FFSRL_ACC_* (0 = fixed point) */
    int32_t precision;       /* 32 (0 means 32) or 64: the float64 build, reference arithmetic */
    int32_t reserved[4];
} ffsrl_batch_options;

/* Build the env-resident batch plan from HOST copies of the model arrays (host_model
   pointers are host memory; sizes and env ranges must be set).  device_model holds the
   device pointers of the same arrays; the plan keeps those for state (vertex, velocity,
   predicted_vertex, drag, instrument) and uploads its own packed constraint tables. */
int32_t ffsrl_batch_create(const ffsrl_model* host_model, const ffsrl_model* device_model,
                           const ffsrl_params* params, const ffsrl_batch_options* opts, ffsrl_batch** out);
int32_t ffsrl_batch_destroy(ffsrl_batch* b);
/* n_steps full steps of every env; same semantics as n_steps ffsrl_step_model calls. */
int32_t ffsrl_batch_step(ffsrl_batch* b, int32_t n_steps, void* stream);
/* Step only the listed envs (HOST array of env ids, count n).  A plan has 2 lanes, each
   with its own work list, counters, scratch and class streams: steps of disjoint env
   sets issued on different lanes (and streams) may run concurrently; the plain call
   uses lane 0.  A lane's previous call must have finished reading its staging buffer,
   which the call waits for. */
int32_t ffsrl_batch_step_envs(ffsrl_batch* b, const int32_t* env_ids, int32_t n, int32_t n_steps, void* stream);
int32_t ffsrl_batch_step_envs_lane(ffsrl_batch* b, int32_t lane, const int32_t* env_ids, int32_t n, int32_t n_steps,
                                   void* stream);
/* bytes of device memory the plan holds; per-env shared-memory class */
int32_t ffsrl_batch_info(const ffsrl_batch* b, int64_t* device_bytes, int32_t* num_classes, int32_t* block_threads);
/* Size classes (environments grouped by vertex count, one launch each): the class's
   largest vertex count, storage mode (0 shared, 1 shared positions + global sums,
   2 global), block size and environment count; its env ids; its block size. */
int32_t ffsrl_batch_class_info(const ffsrl_batch* b, int32_t cls, int32_t* max_nv, int32_t* mode, int32_t* block,
                               int32_t* num_envs);
int32_t ffsrl_batch_class_envs(const ffsrl_batch* b, int32_t cls, int32_t* env_ids);
int32_t ffsrl_batch_set_class_block(ffsrl_batch* b, int32_t cls, int32_t block);
/* Autotuner hook, how class cls's kernel fetches each thread's next tet record one loop
   trip ahead: 0 not at all, 1 into L1 (prefetch.global.L1), 2 into registers (block sizes
   512 and 640, float32).  Results are unchanged.  A kind the class's block size has no
   kernel for is refused and leaves the class as it was. */
int32_t ffsrl_batch_set_class_prefetch(ffsrl_batch* b, int32_t cls, int32_t kind);
/* Copies the float64 plan's state (x, v, predicted, each [3V]) to host memory. */
int32_t ffsrl_batch_state_f64(const ffsrl_batch* b, double* host_xvx);
/* per-env status after a step: 0 ok, FFSRL_ERR_NONFINITE if the env's state went non-finite */
int32_t ffsrl_batch_env_status(const ffsrl_batch* b, int32_t* host_status, int32_t num_envs);

/* ---- owning handle over the batched step ------------------------------------------
   ffsrl_create uploads a model given in HOST memory (an ffsrl_model whose pointers are
   host arrays, sizes as the struct documents) into device arrays the handle owns, and
   builds its batched plan (block_threads 0: automatic).  State and scratch arrays the
   host model leaves NULL (predicted_vertex, velocity, dp, constraints_number,
   collision_dp, lambdas, hole, active_drag_constraint, laparoscope_in_collision) start
   zeroed.  ffsrl_get_device_model fills an ffsrl_model with the device pointers (and the
   plan, for the ffsrl_batch_* calls): callers read and write state, tool and grasp arrays
   there between steps.  ffsrl_set_tool / ffsrl_set_drag copy tool capsules [4N] and the
   grasp mask [V] from host (from_host 1, waits for the copy) or device memory. */
typedef struct ffsrl_handle ffsrl_handle;
int32_t ffsrl_create(const ffsrl_model* host_model, const ffsrl_params* params, int32_t block_threads,
                     ffsrl_handle** handle);
int32_t ffsrl_destroy(ffsrl_handle* handle);
int32_t ffsrl_step(ffsrl_handle* handle, int32_t n_steps, void* stream);
int32_t ffsrl_get_device_model(const ffsrl_handle* handle, ffsrl_model* device_model, ffsrl_batch** plan);
int32_t ffsrl_set_tool(ffsrl_handle* handle, const float* base, const float* tip, const float* radius,
                       int32_t from_host, void* stream);
int32_t ffsrl_set_drag(ffsrl_handle* handle, const float* drag, int32_t from_host, void* stream);

/* Observation for the handle: the visual mesh of all envs in HOST memory (env-major;
   faces hold global point ids within their env's range), remap pairs (visual point,
   simulated vertex) and shading.  ffsrl_attach_render builds one BVH topology per
   distinct env_topology id (NULL: one per env) on its first env's points (the
   reference's binned SAH, 8 bins) and owns every device buffer of the refit and the
   ray-cast.  Texture mode (1) needs texture tables and is not offered here.
   ffsrl_render_handle remaps the visual points from the current vertices, refits and
   ray-casts: color [N*R*R*3] and depth [N*R*R] are caller-owned device arrays; cameras
   are device arrays of 1 or num_envs entries (position [3C], quaternion x,y,z,w [4C]). */
typedef struct {
    int32_t num_points, num_faces;
    const float* points;            /* [3P] visual points, the BVH is built on these */
    const int32_t* faces;           /* [3Fv] */
    const float* colors;            /* [3P] */
    int32_t num_map;
    const int32_t* point_to_vertex; /* [2 * num_map] */
    const int32_t* env_point_start; /* [N+1] */
    const int32_t* env_face_start;  /* [N+1] */
    const int32_t* env_topology;    /* [N] or NULL */
    int32_t resolution;
    float camera_tan, camera_aspect;
    int32_t num_lights;
    const float* light_dir;         /* [3L] */
    const float* light_intensity;   /* [L] */
    int32_t render_mode;            /* 0 grayscale, 2 normal map, 3 vertex colour, 4 depth map */
} ffsrl_render_config;
int32_t ffsrl_attach_render(ffsrl_handle* handle, const ffsrl_render_config* config);
int32_t ffsrl_render_handle(ffsrl_handle* handle, const float* camera_pos, const float* camera_rot, int32_t num_cameras,
                            float* color, float* depth, void* stream);
/* Error state of the handle's ray-casts since the last check (the Python renderer's
   checkErrors, which the reference lacks: its stack is unchecked, render.py:411-498).
   Waits for `stream`, then returns FFSRL_ERR_STACK_OVERFLOW if a ray of a
   ffsrl_render_handle call exhausted its traversal stack (its image then misses that
   ray's hit), and clears the state; FFSRL_OK otherwise.  ffsrl_render_handle itself does
   not wait for the GPU. */
int32_t ffsrl_render_handle_check(ffsrl_handle* handle, void* stream);

/* ---- CUDA graphs (the reference's wp.capture_begin / capture_end / capture_launch,
   bvh.py:442-451, render.py:1108-1112, tests/testLiverRetraction.py:77-85) ----------
   Every launch the library's calls make on `stream` between begin and end is recorded
   (the batched step's class streams join the capture through its fork/join events);
   launch replays them on any stream with the pointers and scalars they were recorded
   with.  The legacy default stream (NULL) cannot be captured.  Calls that wait on the
   host (ffsrl_batch_create, the staged env lists of ffsrl_batch_step_envs) do not belong
   in a capture. */
typedef struct ffsrl_graph ffsrl_graph;
int32_t ffsrl_graph_begin(void* stream);
int32_t ffsrl_graph_end(void* stream, ffsrl_graph** graph);
int32_t ffsrl_graph_launch(const ffsrl_graph* graph, void* stream);
int32_t ffsrl_graph_destroy(ffsrl_graph* graph);

/* ---- serving: continuous batching of RL step requests (admit / evict / submit / poll) --
   Each actor owns one env of a mesh type; envs live in the slots of one batched model,
   slot s holding an env of mesh type slot_mesh[s].  A request is a tool displacement (3
   floats), a clamp flag and a reset flag (the env returns to its rest state first).
   ffsrl_server_launch starts a tick on a free lane with every ready request (its actor
   not in flight; admitted into a free slot of its type, evicting the least recently used
   idle actor of that type when there is none -- its state is kept in host memory and
   restored when it returns).  A tick runs, for exactly those envs: resets, the tool move
   (the kinematic chain when xform is given, else a rigid translation), grasp changes, one
   batched step, the visual remap, the instrument's visual points, the BVH refit and the
   ray-cast.  ffsrl_server_poll returns finished requests: their tags, actors and 4 floats
   each (the drag point tip[4e+3] and the env's contact count).  A lane's tick is returned
   whole, so capacity should be at least num_slots.  Host calls from one thread. */
typedef struct ffsrl_server ffsrl_server;
typedef struct {
    int32_t num_slots;                  /* envs of the model */
    const int32_t* slot_mesh;           /* host [num_slots] mesh type of each slot */
    int32_t num_actors;
    const int32_t* actor_mesh;          /* host [num_actors] mesh type of each actor's env */
    int32_t lanes;                      /* ticks in flight at once: 1 or 2 (the plan's lanes) */
    ffsrl_batch* plan;                  /* the model's batched plan */
    const ffsrl_model* model;           /* device arrays of the model (copied at create) */
    const float* initial_vertex;        /* [3V] rest state */
    const float* initial_base;          /* [3*4N] */
    const float* initial_tip;           /* [3*4N] */
    float* xform;                       /* [112N] instrument transforms, or NULL */
    const float* initial_xform;         /* [112N] (with xform) */
    const float* height;                /* [4N] capsule heights (with xform) */
    const int32_t* grasp_cand_start;    /* [N+1] grasp candidates of each env */
    const int32_t* grasp_cand;
    float grasp_radius;                 /* drag lookup radius */
    float* vis_point;                   /* all visual points */
    const int32_t* point_to_vertex;     /* remap pairs */
    const int32_t* env_map_start;       /* [N+1] */
    const float* inst_local_point;      /* instrument visual mesh (inst_num_points 0: none) */
    const int32_t* inst_point_slot;
    int32_t inst_num_points;
    const int32_t* env_inst_first_point;/* [N] */
    const ffsrl_bvh* bvh;               /* copied at create */
    const int32_t* vis_face;
    const ffsrl_render* render;         /* copied at create */
} ffsrl_server_config;
int32_t ffsrl_server_create(const ffsrl_server_config* config, ffsrl_server** server);
int32_t ffsrl_server_destroy(ffsrl_server* server);
int32_t ffsrl_server_submit(ffsrl_server* server, int32_t actor, const float* disp, int32_t clamp, int32_t reset,
                            int64_t tag);
/* starts a tick of at most max_batch requests (<= 0: no limit); *launched = its size */
int32_t ffsrl_server_launch(ffsrl_server* server, int32_t max_batch, int32_t* launched);
int32_t ffsrl_server_poll(ffsrl_server* server, int32_t capacity, int64_t* tags, int32_t* actors, float* results,
                          int32_t* count);
/* explicit admission (returns the slot; FFSRL_ERR_BUSY when every slot of the type is in
   flight) and eviction (FFSRL_ERR_BUSY while the actor's tick is not polled) */
int32_t ffsrl_server_admit(ffsrl_server* server, int32_t actor, int32_t* slot);
int32_t ffsrl_server_evict(ffsrl_server* server, int32_t actor);
int32_t ffsrl_server_stats(const ffsrl_server* server, int64_t* admissions, int64_t* evictions, int32_t* pending,
                           int32_t* in_flight);

/* ---- cutting and heating (integrator.py:700-918, 1153-1185, 1406-1518, 1583-1605) ----
   Library calls over the env-major arrays; the reference's DO step does not launch them.
   One thread per element.  Element maps use -1 for "none" (no neighbour, no surface
   triangle) and such entries are skipped.  Instrument points are the capsule tips
   [3 * 4 * num_envs] (entry 4e+k of env e: k = 0 rod, 1 and 2 the clamps); an element's
   env comes from an optional element -> env map (NULL: env 0, the reference's single
   instrument).  An optional env_tet_start [num_envs + 1] with that map limits a tet scan
   to the edge's env, which gives the result of the reference's scan over all tets. */
/* edgeBreakerKernel (integrator.py:700-731): an edge with active_edge != 0, rest length
   and current length both at least 2.22e-16, and stretch C = len / rest - 1 above
   break_threshold adds (C - break_threshold) * break_factor to breaker_value[e]. */
int32_t ffsrl_edge_breaker(const float* predicted, const int32_t* edge, const float* rest_length,
                           const float* active_edge, float* breaker_value, int32_t num_edges, float break_factor,
                           float break_threshold, void* stream);
/* checkEdgeBreakerKernel (integrator.py:733-775): an edge whose breaker value exceeds
   break_limit gets flip_edges[e] = -1 (if 0 and active == 1), opens the surface triangles
   edge_to_triangles[2e], [2e+1] (holes[f] = 1) and, where some tet holds both its
   vertices, sets flip_tets[e] = -1 if flip_tets[e] is 0 and active_tet[e] is 1.  The
   reference indexes the tet flags by the EDGE id; edges with ids >= num_tets skip that
   part. */
int32_t ffsrl_check_edge_breaker(const float* breaker_value, const int32_t* edge, const float* active_edge,
                                 int32_t* flip_edges, int32_t num_edges, const int32_t* tetrahedron, int32_t num_tets,
                                 const float* active_tet, int32_t* flip_tets, const int32_t* edge_to_triangles,
                                 int32_t* holes, float break_limit, const int32_t* edge_to_env,
                                 const int32_t* env_tet_start, void* stream);
/* tetrahedronBreaker (integrator.py:777-818): a tet with active == 1 whose signed volume
   exceeds its rest volume adds (volume - rest) * break_factor to breaker_value[t].
   tetrahedron is [4T] (the reference's four per-corner arrays interleaved). */
int32_t ffsrl_tetrahedron_breaker(const float* predicted, const int32_t* tetrahedron, const float* rest_volume,
                                  const float* active_tet, float* breaker_value, int32_t num_tets,
                                  float break_factor, void* stream);
/* tetrahedronHeatPropagation (integrator.py:820-847): for a tet with active != 0,
   new_heat[t] = h (1 - loss) + transfer * sum over active neighbours n of (h_n - h) conduction.
   neighbors is [4T], entry i the tet across the face opposite vertex i, or -1. */
int32_t ffsrl_heat_propagation(const float* active_tet, const int32_t* neighbors, const float* heat,
                               float* new_heat, int32_t num_tets, float conduction, float transfer, float loss,
                               void* stream);
/* tetrahedronHeatUpdate (integrator.py:849-872): heat[t] = new_heat[t] for active tets
   (0 otherwise); each vertex of an active tet takes heat / 4 from the highest-id active
   tet holding it, the last writer of a serial run.  owner_scratch is num_vertices ints
   of device scratch. */
int32_t ffsrl_heat_update(float* heat, const float* new_heat, const float* active_tet, const int32_t* tetrahedron,
                          float* vertex_heat, int32_t* owner_scratch, int32_t num_tets, int32_t num_vertices,
                          void* stream);
/* checkTetrahedronHeat (integrator.py:874-895) with rest_volume NULL: heat > heat_limit
   and flip_tets[t] == 0 set flip_tets[t] = -1 and open the tet's surface triangles
   tet_to_triangles[4t..4t+3].  checkTetrahedronHeatVolumeProportional
   (integrator.py:897-918) with rest_volume: heat > heat_limit * rest_volume[t] does the
   same whatever flip_tets[t] was. */
int32_t ffsrl_check_heat(const float* heat, int32_t* flip_tets, const float* rest_volume,
                         const int32_t* tet_to_triangles, int32_t* holes, float heat_limit, int32_t num_tets,
                         void* stream);
/* heatLaparoscope (integrator.py:1153-1185): each surface triangle whose closest point to
   the midpoint of its env's clamp tips (entries 4e+1, 4e+2) lies within sphere_radius adds
   heat_quantum to its tet triangle_to_tet[f] if that tet is active. */
int32_t ffsrl_heat_laparoscope(const int32_t* triangle, const float* positions, const float* active_tet, float* heat,
                               const int32_t* triangle_to_tet, const float* capsule_tips,
                               const int32_t* triangle_to_env, float sphere_radius, float heat_quantum,
                               int32_t num_triangles, void* stream);
/* findIntersectingEdges (integrator.py:1406-1458) with checkSegmentTriangleIntersection
   (integrator.py:1471-1518): an edge crossing the triangle (rod tip, right clamp tip,
   left clamp tip) of its env gets flip_edges[e] = -1 (if 0 and active == 1), opens its
   surface triangles, and flips (-1) every tet holding both its vertices whose flag is 0
   and whose active value is 1. */
int32_t ffsrl_cut_edges(const float* positions, const float* capsule_tips, const int32_t* edge,
                        const float* active_edge, int32_t* flip_edges, int32_t num_edges, const int32_t* tetrahedron,
                        int32_t num_tets, const float* active_tet, int32_t* flip_tets,
                        const int32_t* edge_to_triangles, int32_t* holes, const int32_t* edge_to_env,
                        const int32_t* env_tet_start, void* stream);
/* inDeCreaseActiveValues (integrator.py:1583-1605): element t with flip f != 0 takes
   active = table[f] (f > 0, then f + 1) or table[steps + f] (f < 0, then f - 1), and
   the counter returns to 0 once |f| >= steps.  table holds steps + 1 values (the
   reference: sqrt(k / 5), k = 0..5).  Counters with |f| > steps are left alone. */
int32_t ffsrl_update_active_values(int32_t* flip, float* active, const float* table, int32_t steps, int32_t n,
                                   void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FFSRL_H */
