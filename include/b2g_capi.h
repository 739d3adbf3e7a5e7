/*
 * b2g_capi.h - C ABI of the GB300 Step engine (box2d-optimized_gb300).
 *
 * One shared library, libb2g.so, steps batches of Box2D worlds on one GPU. The ABI takes plain
 * pointers, sizes and POD structs; no C++ or torch types cross it; every entry point returns an
 * int status (B2G_OK or a B2G_E* code) and never throws.
 *
 * Each entry point replaces one piece of the reference's public C++ API (file:line cited beside
 * it). The C++ facade in box2d-optimized_gb300/include/box2d/ (b2World, b2Body, b2Fixture,
 * b2Joint, b2Contact) is written on top of these calls.
 *
 * Threading: one host thread per batch handle. A batch may hold many independent worlds; a world
 * is addressed by (batch, world index). Bodies, fixtures and joints are addressed by their
 * creation index inside their world.
 */
#ifndef B2G_CAPI_H
#define B2G_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define B2G_API __declspec(dllexport)
#else
#define B2G_API __attribute__((visibility("default")))
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define B2G_OK 0
#define B2G_E_INVALID_ARG 1   /* bad handle, index, size or malformed definition            */
#define B2G_E_OUT_OF_MEMORY 2 /* host or device allocation failed / budget exceeded          */
#define B2G_E_TIMEOUT 3       /* a bounded device wait ran out (the step did not complete)   */
#define B2G_E_WORLD_FAULT 4   /* a world produced a non-finite state and was frozen          */
#define B2G_E_CUDA 5          /* a CUDA runtime call failed (no device, launch error, ...)    */
#define B2G_E_LOCKED 6        /* world is locked (inside a step)                              */
#define B2G_E_CAPACITY 7      /* a fixed-size buffer is too small for the request            */
#define B2G_E_CANCELLED 8     /* a served request was cancelled before it finished            */

/* ---- enums mirroring the reference's values ---------------------------------------------- */
/* b2BodyType, include/box2d/b2_body.h:44-49 */
#define B2G_STATIC 0
#define B2G_KINEMATIC 1
#define B2G_DYNAMIC 2
/* b2Shape::Type, include/box2d/b2_shape.h:52-59 */
#define B2G_SHAPE_CIRCLE 0
#define B2G_SHAPE_EDGE 1
#define B2G_SHAPE_POLYGON 2
/* b2JointType, include/box2d/b2_joint.h:35-49 (gear and rope joints are not supported) */
#define B2G_JOINT_REVOLUTE 1
#define B2G_JOINT_PRISMATIC 2
#define B2G_JOINT_DISTANCE 3
#define B2G_JOINT_PULLEY 4
#define B2G_JOINT_MOUSE 5
#define B2G_JOINT_WHEEL 7
#define B2G_JOINT_WELD 8
#define B2G_JOINT_FRICTION 9
#define B2G_JOINT_MOTOR 11
#define B2G_JOINT_GEAR 6
/* b2Manifold::Type, include/box2d/b2_collision.h:105-110 */
#define B2G_MANIFOLD_CIRCLES 0
#define B2G_MANIFOLD_FACE_A 1
#define B2G_MANIFOLD_FACE_B 2

#define B2G_MAX_POLYGON_VERTICES 8 /* b2_maxPolygonVertices, b2_settings.h:54 */

/* ---- geometry ----------------------------------------------------------------------------- */
/* A processed shape in its body frame (b2CircleShape / b2EdgeShape / b2PolygonShape state).
 *   circle : vertices[0] = m_p, radius = m_radius
 *   edge   : vertices[0] = m_vertex1, [1] = m_vertex2, [2] = m_vertex0, [3] = m_vertex3,
 *            one_sided = m_oneSided, radius = b2_polygonRadius
 *   polygon: vertices/normals[0..count), centroid = m_centroid, radius = b2_polygonRadius   */
typedef struct b2g_shape {
  int32_t type;
  int32_t count;
  float radius;
  int32_t one_sided;
  float vertices[B2G_MAX_POLYGON_VERTICES][2];
  float normals[B2G_MAX_POLYGON_VERTICES][2];
  float centroid[2];
} b2g_shape; /* 152 bytes */

/* b2ManifoldPoint (b2_collision.h:75-85): 20 bytes. id = b2ContactID.key, i.e.
 * indexA | indexB << 8 | typeA << 16 | typeB << 24. */
typedef struct b2g_manifold_point {
  float local_point[2];
  float normal_impulse;
  float tangent_impulse;
  uint32_t id;
} b2g_manifold_point;

/* b2Manifold (b2_collision.h:103-117): 64 bytes, same field meaning and order. */
typedef struct b2g_manifold {
  b2g_manifold_point points[2];
  float local_normal[2];
  float local_point[2];
  int32_t type;
  int32_t point_count;
} b2g_manifold;

/* b2Sweep (include/box2d/b2_math.h:383-404): 36 bytes, same fields in the same order. */
typedef struct b2g_sweep {
  float local_center[2];
  float c0[2];
  float c[2];
  float a0;
  float a;
  float alpha0;
} b2g_sweep;

/* b2TOIInput (include/box2d/b2_time_of_impact.h:29-36): the two b2DistanceProxy are given as
 * their shapes (a circle's proxy is its centre, an edge's its two vertices, a polygon's its
 * vertices; the radius is the shape's). */
typedef struct b2g_toi_input {
  b2g_shape shape_a;
  b2g_shape shape_b;
  b2g_sweep sweep_a;
  b2g_sweep sweep_b;
  float t_max;
} b2g_toi_input;

/* b2TOIOutput::State (include/box2d/b2_time_of_impact.h:42-49) */
#define B2G_TOI_UNKNOWN 0
#define B2G_TOI_FAILED 1
#define B2G_TOI_OVERLAPPED 2
#define B2G_TOI_TOUCHING 3
#define B2G_TOI_SEPARATED 4
typedef struct b2g_toi_output {
  int32_t state;
  float t;
} b2g_toi_output;

/* ---- definitions (inputs) ------------------------------------------------------------------ */
/* b2BodyDef, include/box2d/b2_body.h:52-130 */
typedef struct b2g_body_def {
  int32_t type;
  float position[2];
  float angle;
  float linear_velocity[2];
  float angular_velocity;
  float linear_damping;
  float angular_damping;
  float gravity_scale;
  int32_t allow_sleep;
  int32_t awake;
  int32_t fixed_rotation;
  int32_t bullet;
  int32_t enabled;
  uint64_t user_data;
} b2g_body_def;

/* How a polygon fixture's geometry is given. */
#define B2G_POLY_HULL 0       /* b2PolygonShape::Set(vertices, count)          b2_polygon_shape.cpp:113 */
#define B2G_POLY_BOX 1        /* b2PolygonShape::SetAsBox(hx, hy)               b2_polygon_shape.cpp:36  */
#define B2G_POLY_BOX_ORIENTED 2 /* SetAsBox(hx, hy, center, angle)              b2_polygon_shape.cpp:50  */
#define B2G_POLY_RAW 3        /* already-processed b2g_shape given in `shape`                           */

/* b2FixtureDef (include/box2d/b2_fixture.h:60-110) with its shape given inline. */
typedef struct b2g_fixture_def {
  int32_t body;         /* creation index of the owning body in the same world */
  int32_t shape_type;   /* B2G_SHAPE_* */
  int32_t poly_mode;    /* B2G_POLY_* for polygons */
  int32_t count;        /* raw vertex count for B2G_POLY_HULL */
  float verts[B2G_MAX_POLYGON_VERTICES][2]; /* hull input; edge: v1, v2, v0, v3 */
  float box[5];         /* hx, hy, center.x, center.y, angle */
  float radius;         /* circle radius */
  float center[2];      /* circle m_p */
  int32_t one_sided;    /* edge */
  float friction;
  float restitution;
  float restitution_threshold;
  float density;
  int32_t is_sensor;
  uint16_t category_bits;
  uint16_t mask_bits;
  int16_t group_index;
  int16_t pad0;
  uint64_t user_data;
  b2g_shape shape;      /* B2G_POLY_RAW input */
} b2g_fixture_def;

/* The joint definitions in one record: b2RevoluteJointDef (b2_revolute_joint.h:39-88),
 * b2PrismaticJointDef (b2_prismatic_joint.h:35-88), b2DistanceJointDef (b2_distance_joint.h:33-70),
 * b2WeldJointDef (b2_weld_joint.h:31-65), b2WheelJointDef (b2_wheel_joint.h:34-89),
 * b2MotorJointDef (b2_motor_joint.h:29-59), b2FrictionJointDef (b2_friction_joint.h:29-56),
 * b2MouseJointDef (b2_mouse_joint.h:30-56), b2PulleyJointDef (b2_pulley_joint.h:32-75),
 * b2GearJointDef (b2_gear_joint.h:28-45). A mouse joint's local_anchor_b is computed from its
 * target when it is created, as the reference's constructor does. A gear joint names two earlier
 * revolute or prismatic joints of its world (joint_1, joint_2) and a ratio; on creation the engine
 * takes its bodies from them (body_a = joint 1's body B, body_b = joint 2's body B, as
 * b2GearJoint::b2GearJoint does, src/dynamics/b2_gear_joint.cpp:48-139) and stores the gear's
 * constant (coordinate 1 + ratio * coordinate 2 at creation) in gear_constant. */
typedef struct b2g_joint_def {
  int32_t type;             /* B2G_JOINT_* */
  int32_t body_a;
  int32_t body_b;
  int32_t collide_connected;
  float local_anchor_a[2];
  float local_anchor_b[2];
  float reference_angle;    /* revolute, prismatic, weld; motor: angularOffset */
  float local_axis_a[2];    /* prismatic (normalised on creation), wheel (as given) */
  int32_t enable_limit;
  float lower;              /* lowerAngle / lowerTranslation */
  float upper;              /* upperAngle / upperTranslation */
  int32_t enable_motor;
  float max_motor;          /* maxMotorTorque / maxMotorForce */
  float motor_speed;
  float length;             /* distance */
  float min_length;
  float max_length;
  float stiffness;          /* distance, weld, wheel, mouse */
  float damping;
  float linear_offset[2];   /* motor */
  float max_force;          /* motor, friction, mouse */
  float max_torque;         /* motor, friction */
  float correction_factor;  /* motor */
  float target[2];          /* mouse: world target point */
  float ground_anchor_a[2]; /* pulley */
  float ground_anchor_b[2];
  float length_a, length_b; /* pulley rope lengths */
  float ratio;              /* pulley, gear */
  uint64_t user_data;
  int32_t joint_1, joint_2; /* gear: the joints it couples (indices in the world) */
  float gear_constant;      /* gear: set on creation */
  int32_t reserved;
} b2g_joint_def;

/* ---- state records (outputs / snapshot) ------------------------------------------------------ */
/* Body state and mass data (b2Body members, include/box2d/b2_body.h:480-560). */
#define B2G_BODY_ENABLED 1u
#define B2G_BODY_FIXED_ROTATION 2u
#define B2G_BODY_BULLET 4u
#define B2G_BODY_AWAKE 8u
#define B2G_BODY_AUTO_SLEEP 16u
typedef struct b2g_body {
  float xf[4];             /* m_xf: p.x, p.y, q.s, q.c */
  float c[2];              /* m_sweep.c */
  float a;                 /* m_sweep.a */
  float v[2];              /* m_linearVelocity */
  float w;                 /* m_angularVelocity */
  float local_center[2];   /* m_sweep.localCenter */
  float mass, inv_mass, inertia, inv_inertia;
  float linear_damping, angular_damping, gravity_scale;
  float force[2];
  float torque;
  int32_t type;
  uint32_t flags;
} b2g_body; /* 96 bytes */

typedef struct b2g_fixture {
  b2g_shape shape;
  int32_t body;
  float density, friction, restitution, restitution_threshold;
  uint16_t category_bits, mask_bits;
  int16_t group_index;
  uint8_t is_sensor;
  uint8_t pad0;
} b2g_fixture;

/* Joint parameters and warm-start state. impulse[0..2]: revolute m_impulse (x, y), prismatic
 * m_impulse (x, y), distance m_impulse in [0]. */
/* impulse[]: revolute / prismatic m_impulse (x, y), distance and pulley m_impulse in [0], weld
 * m_impulse (x, y, z), wheel (m_impulse, m_springImpulse), motor and friction (linear x, y,
 * angular), mouse m_impulse (x, y), gear m_impulse in [0]. */
typedef struct b2g_joint {
  b2g_joint_def def;
  float impulse[3];
  float motor_impulse, lower_impulse, upper_impulse;
  float reaction_impulse[2];      /* GetReactionForce(inv_dt) / inv_dt after the last step */
  float reaction_angular_impulse; /* GetReactionTorque(inv_dt) / inv_dt after the last step */
} b2g_joint;

/* b2Contact (include/box2d/b2_contact.h:155-173 flags) */
#define B2G_CONTACT_TOUCHING 2u
#define B2G_CONTACT_ENABLED 4u
typedef struct b2g_contact {
  int32_t fixture_a;       /* creation index of fixture A in its world */
  int32_t fixture_b;
  uint32_t flags;
  float friction, restitution, restitution_threshold, tangent_speed;
  b2g_manifold manifold;
} b2g_contact;

/* Listener events (b2ContactListener, b2_world_callbacks.h:133-209), delivered as a batch after
 * each step in the order: End (contacts destroyed by the broadphase), Begin, End, PreSolve
 * (from the narrowphase), PostSolve (from the solver). */
#define B2G_EVENT_BEGIN 1
#define B2G_EVENT_END 2
#define B2G_EVENT_PRESOLVE 3
#define B2G_EVENT_POSTSOLVE 4
typedef struct b2g_event {
  int32_t kind;
  int32_t world;
  int32_t fixture_a;
  int32_t fixture_b;
  int32_t point_count;     /* PostSolve: b2ContactImpulse::count */
  float normal_impulses[2];
  float tangent_impulses[2];
  b2g_manifold old_manifold; /* PreSolve: the manifold before this step's update */
} b2g_event;

/* b2Profile (include/box2d/b2_time_step.h:29-36), milliseconds of the last step (device time). */
typedef struct b2g_profile {
  float step, collide, solve, broadphase, solve_toi;
  int64_t bodies, fixtures, contacts, touching, joints, colors_max;
  int64_t touching_total; /* solver contacts summed over every step of the batch so far */
  /* host wall times of the last b2g_step (ms): the whole call; uploading appended worlds; their
   * broadphase (with its read-back); growing device buffers */
  float host_step, host_admit_upload, host_admit_broadphase, host_grow;
} b2g_profile;

/* ---- batch lifecycle ------------------------------------------------------------------------ */
typedef struct b2g_batch b2g_batch;

/* Device memory budget in bytes (0 = no limit). Allocation beyond it fails with
 * B2G_E_OUT_OF_MEMORY instead of reaching cudaMalloc. device = B2G_HOST_ONLY makes a batch
 * that builds, edits and reads worlds on the host but cannot step (no GPU needed). */
#define B2G_HOST_ONLY (-1)
B2G_API int b2g_batch_create(int device, uint64_t budget_bytes, b2g_batch** out);
B2G_API int b2g_batch_destroy(b2g_batch* b);

/* b2World::b2World(gravity), include/box2d/b2_world.h:54 */
B2G_API int b2g_world_add(b2g_batch* b, float gx, float gy, int32_t* out_world);
B2G_API int b2g_world_count(b2g_batch* b, int32_t* out_n);
/* b2World::SetGravity / SetAllowSleeping / SetWarmStarting / SetContinuousPhysics /
 * SetAutoClearForces, include/box2d/b2_world.h:195-235. With continuous physics on and a bullet
 * or kinematic body in the world, each step ends with b2World::SolveTOI (src/dynamics/
 * b2_world.cpp:859-1106) on the device, followed by a second pair update. The world's default
 * (b2g_world_add) is off; the b2World facade turns it on, as the reference's constructor does. */
B2G_API int b2g_world_set_gravity(b2g_batch* b, int32_t world, float gx, float gy);
B2G_API int b2g_world_set_flags(b2g_batch* b, int32_t world, int32_t allow_sleep,
                                int32_t warm_starting, int32_t continuous, int32_t auto_clear_forces);
/* The world's flags as b2g_world_set_flags last set them (b2World::GetAllowSleeping,
 * GetWarmStarting, GetContinuousPhysics, GetAutoClearForces). */
B2G_API int b2g_world_get_flags(b2g_batch* b, int32_t world, int32_t* allow_sleep, int32_t* warm_starting,
                                int32_t* continuous, int32_t* auto_clear_forces);

/* b2World::CreateBody, include/box2d/b2_world.h:80 (bulk). out_ids may be NULL. */
B2G_API int b2g_bodies_add(b2g_batch* b, int32_t world, const b2g_body_def* defs, int32_t n,
                           int32_t* out_ids);
/* b2Body::CreateFixture, src/dynamics/b2_body.cpp:230 (bulk; runs ResetMassData per body). */
B2G_API int b2g_fixtures_add(b2g_batch* b, int32_t world, const b2g_fixture_def* defs, int32_t n,
                             int32_t* out_ids);
/* b2World::CreateJoint, src/dynamics/b2_world.cpp:268 (bulk). */
B2G_API int b2g_joints_add(b2g_batch* b, int32_t world, const b2g_joint_def* defs, int32_t n,
                           int32_t* out_ids);

/* Checkpoint / resume. b2g_world_snapshot writes one world's complete state (bodies, fixtures,
 * joints with their warm-start impulses, the live contacts with their manifolds and impulses,
 * gravity, the previous step's inverse time step, flags) into buf as a self-describing blob of
 * *size bytes (pass cap = 0 to learn the size: B2G_E_CAPACITY). b2g_world_restore appends such a
 * world to a batch (any batch); stepping it continues bit-identically to the original. A
 * restore re-lays out the batch at its next step. (The reference has b2World::Dump,
 * src/dynamics/b2_world.cpp:1469-1531, which writes C++ code and no contacts; this is the
 * binary resume it lacks.) */
B2G_API int b2g_world_snapshot(b2g_batch* b, int32_t world, void* buf, uint64_t cap, uint64_t* size);
B2G_API int b2g_world_restore(b2g_batch* b, const void* buf, uint64_t size, int32_t* out_world);
/* Whether a world is still stepped: *status = B2G_E_WORLD_FAULT once a step left one of its
 * bodies with a non-finite position or velocity. Such a world is frozen (no later step touches
 * it; its last state stays readable) while the other worlds of the batch go on. */
B2G_API int b2g_world_status(b2g_batch* b, int32_t world, int32_t* status);
/* Retires a world (it is no longer stepped; its contacts go at the next broadphase) and
 * b2g_compact removes retired worlds, writing each old index's new index (-1 = removed) into
 * old_to_new. (The reference's b2World destructor, src/dynamics/b2_world.cpp:71-101, for worlds
 * that share a batch.) */
B2G_API int b2g_world_retire(b2g_batch* b, int32_t world);
B2G_API int b2g_compact(b2g_batch* b, int32_t* old_to_new, int32_t n);

/* Counts of one world. */
/* b2World::Dump (src/dynamics/b2_world.cpp:1469-1531): the world as C++ source that rebuilds it
 * through the b2World API, in the reference's text format (same lines and order, %.9g numbers).
 * Writes up to cap - 1 characters and a terminating zero to `out`; *n receives the text's length,
 * and B2G_E_CAPACITY is returned when it does not fit (call with cap = 0 to size the buffer). */
B2G_API int b2g_world_dump(b2g_batch* b, int32_t world, char* out, uint64_t cap, uint64_t* n);
/* Structural removal: b2World::DestroyBody (src/dynamics/b2_world.cpp:178-266), b2Body::DestroyFixture
 * (src/dynamics/b2_body.cpp:280-350), b2World::DestroyJoint (b2_world.cpp:326-410). A removed body
 * takes its fixtures, joints and contacts along; a destroyed contact that was touching ends, and the
 * End events are returned at once in `ended` (up to `cap`; *n_ended = their number, fixture indices
 * from before the removal), as the reference calls EndContact inside the destroy call; a destroyed
 * contact with manifold points wakes both bodies, a removed joint wakes its bodies, a removed fixture
 * resets its body's mass data. The remaining bodies, fixtures and joints of the world keep their
 * creation order and are renumbered from 0; the world is re-uploaded by its next step and its other
 * contacts keep their manifolds and impulses. */
B2G_API int b2g_bodies_remove(b2g_batch* b, int32_t world, const int32_t* bodies, int32_t n, b2g_event* ended,
                              int32_t cap, int32_t* n_ended);
B2G_API int b2g_fixtures_remove(b2g_batch* b, int32_t world, const int32_t* fixtures, int32_t n,
                                b2g_event* ended, int32_t cap, int32_t* n_ended);
B2G_API int b2g_joints_remove(b2g_batch* b, int32_t world, const int32_t* joints, int32_t n);
B2G_API int b2g_world_sizes(b2g_batch* b, int32_t world, int32_t* bodies, int32_t* fixtures,
                            int32_t* joints, int32_t* contacts);

/* ---- stepping ------------------------------------------------------------------------------- */
/* b2World::Step(dt, velocityIterations, positionIterations), include/box2d/b2_world.h:127-141,
 * for every world of the batch whose world_mask entry is non-zero (world_mask NULL = all).
 * Returns after the step's device work has been enqueued and completed. */
B2G_API int b2g_step(b2g_batch* b, float dt, int32_t velocity_iterations,
                     int32_t position_iterations, const uint8_t* world_mask);
/* b2g_step in two halves, so that host work (building worlds, b2g_batch_stage) overlaps the
 * device's step: b2g_step_begin uploads and launches the step and returns; b2g_step_poll reports
 * whether the device has finished it (non-blocking); b2g_step_end waits and completes it (status
 * as b2g_step). Between them only worlds that are not on the device yet may be created or edited
 * and b2g_batch_stage called; other calls on the batch return B2G_E_LOCKED. */
B2G_API int b2g_step_begin(b2g_batch* b, float dt, int32_t velocity_iterations, int32_t position_iterations,
                           const uint8_t* world_mask);
B2G_API int b2g_step_poll(b2g_batch* b, int32_t* done);
B2G_API int b2g_step_end(b2g_batch* b);
/* Packs the worlds added since the last step into device layout on the host (no device work), so
 * that the next step's upload of them is a copy; call it while a step runs. Edits to those worlds
 * afterwards discard the pack (the next step then packs them itself). */
B2G_API int b2g_batch_stage(b2g_batch* b);
/* n steps back to back; with use_graph != 0 the whole Step is captured once in a CUDA graph and
 * replayed (buffers are sized on the first step; see b2g_reserve). */
B2G_API int b2g_step_n(b2g_batch* b, float dt, int32_t velocity_iterations,
                       int32_t position_iterations, int32_t n, int32_t use_graph);
/* n steps back to back, timed with CUDA events recorded on the engine's stream around them;
 * *device_ms receives the elapsed device time (all n steps). */
B2G_API int b2g_step_timed(b2g_batch* b, float dt, int32_t velocity_iterations,
                           int32_t position_iterations, int32_t n, float* device_ms);
/* Host -> device copy of the force and torque of every body of the batch (device order = world,
 * then creation order): f4 holds (fx, fy, torque, unused) per body, n_bodies records. The
 * per-step input of an end-to-end loop (b2Body::ApplyForce / ApplyTorque on every body). */
B2G_API int b2g_batch_set_forces(b2g_batch* b, const float* f4, int64_t n_bodies);
/* One Step of every world with its host input and output (the end-to-end loop of a driver:
 * b2Body::ApplyForce / ApplyTorque on every body, b2World::Step src/dynamics/b2_world.cpp:1108-1171,
 * b2Body::GetTransform on every body): f4 as b2g_batch_set_forces (NULL: the forces already set),
 * xf4_out as b2g_batch_read_states' xf4 (NULL: none; *n_out receives the bodies). The results equal
 * b2g_batch_set_forces + b2g_step + b2g_batch_read_states; the copies run on a stream of their own,
 * the forces' while the contacts are updated (they are needed from the velocity integration on)
 * and the transforms' while the closing broadphase runs. Synchronous: returns after the step and
 * both copies. Pinned host buffers give the copies their full bandwidth. */
B2G_API int b2g_step_io(b2g_batch* b, float dt, int32_t velocity_iterations, int32_t position_iterations,
                        const float* f4, int64_t n_bodies, float* xf4_out, int64_t cap_bodies, int64_t* n_out);
/* Whether b2g_step replays the Step as a captured CUDA graph (default on). A graph is used for
 * unmasked steps with dt > 0 and events off; it is re-captured when buffers move. */
B2G_API int b2g_batch_set_graphs(b2g_batch* b, int32_t enable);
/* Debug checks (default off): after every solve, a device pass verifies that no regular colour
 * of the constraint colouring holds two contacts or two joints on the same non-static body, and,
 * in worlds that track sleep, that the step's island labels are consistent (each a root, and
 * solid contacts and joints within one island); a violation makes the step return
 * B2G_E_CAPACITY with a message. Costs one small launch per step. No reference counterpart (the
 * reference solves serially). */
B2G_API int b2g_batch_set_debug_checks(b2g_batch* b, int32_t enable);
/* Threads per world CTA of the solver for each world size class (worlds of at most 64, 512,
 * 2048 and 8192 bodies, and larger), 5 entries each one of 64, 128, 256, 512, 1024 (defaults
 * 64, 128, 256, 512, 1024). A tuning knob: results do not depend on it. No reference counterpart. */
B2G_API int b2g_batch_set_solver_threads(b2g_batch* b, const int32_t* threads);
B2G_API int b2g_batch_get_solver_threads(b2g_batch* b, int32_t* threads);
/* The solver kernel comes in two builds: one for occupancy (1024 threads per SM, at most 64
 * registers a thread) and a wide one (512 threads per SM, up to 128 registers, unspilled) whose
 * per-world solve is faster. A size class runs the wide build when its worlds fill at most
 * `waves` waves of it (default: every class; 0 never). A tuning knob: results do not depend on it. */
B2G_API int b2g_batch_set_solver_waves(b2g_batch* b, float waves);
/* Worlds of more than 8192 bodies (single large scenes) are solved by a thread-block cluster of
 * `ctas` CTAs of 512 threads each, one world per cluster, so that one world's colours run on
 * that many SMs at once (the reference solves one island at a time on one core,
 * src/dynamics/b2_world.cpp:526-647). ctas: -1 (default) the largest cluster the device runs
 * (16, else 8); 2, 4, 8 or 16 (capped at that); 0 or 1 one CTA per world. A tuning knob: results
 * do not depend on it. No reference counterpart. */
B2G_API int b2g_batch_set_cluster_solve(b2g_batch* b, int32_t ctas);
/* The CTAs per world that the batch's worlds above 8192 bodies are solved with (1: one CTA). */
B2G_API int b2g_batch_get_cluster_solve(b2g_batch* b, int32_t* ctas);
/* The broadphase keeps each world's tree between steps and refits its boxes; every `period`
 * broadphases (default 32; 1 = every one) it rebuilds all trees from sorted Morton codes, which
 * restores their spatial order. A tuning knob: the pairs found, and so the results, do not
 * depend on it. */
B2G_API int b2g_batch_set_tree_rebuild_period(b2g_batch* b, int32_t period);
/* Autotuner: picks each size class's threads per world by timing the solver over `steps` eager
 * steps per candidate (the class's current count, half and double), largest worlds first. The
 * steps are real steps of the batch (its worlds advance; their number goes to steps_taken);
 * results are bit-identical whatever it picks. Writes the chosen counts to threads_out (5
 * entries) when not null. No reference counterpart. */
B2G_API int b2g_batch_autotune(b2g_batch* b, int32_t steps, float dt, int32_t velocity_iterations,
                               int32_t position_iterations, int32_t* threads_out, int32_t* steps_taken);
/* Testing knob: sets the contact/pair buffer capacity to exactly `cap` (>= live contacts), so
 * that a later broadphase overflows and exercises the recovery path. */
B2G_API int b2g_debug_set_contact_capacity(b2g_batch* b, int64_t cap);
/* Pre-size the pair/contact buffers to at least `contacts` entries in total. */
B2G_API int b2g_reserve(b2g_batch* b, int64_t contacts);

/* ---- reading and writing state ---------------------------------------------------------------- */
/* b2Body getters (GetPosition, GetAngle, GetLinearVelocity, ...), include/box2d/b2_body.h:141-260 */
B2G_API int b2g_bodies_read(b2g_batch* b, int32_t world, int32_t first, int32_t n, b2g_body* out);
/* b2Body::SetTransform / SetLinearVelocity / SetAngularVelocity / ApplyForce...,
 * src/dynamics/b2_body.cpp:482 (writes xf, sweep, velocities, force and torque of each record; a
 * non-zero velocity wakes the body and restarts its sleep timer, as SetLinearVelocity does) */
B2G_API int b2g_bodies_write(b2g_batch* b, int32_t world, int32_t first, int32_t n,
                             const b2g_body* in);
/* b2Body::SetAwake (include/box2d/b2_body.h:719-740): awake = 0 puts the body to sleep (velocity,
 * force and torque cleared); a static body ignores it. */
B2G_API int b2g_body_set_awake(b2g_batch* b, int32_t world, int32_t body, int32_t awake);
/* b2Body::SetBullet (include/box2d/b2_body.h:701-711): the body takes part in continuous
 * collision with other dynamic bodies (B2G_BODY_BULLET in b2g_body.flags). */
B2G_API int b2g_body_set_bullet(b2g_batch* b, int32_t world, int32_t body, int32_t bullet);
/* The bodies' sleep timers (b2Body::m_sleepTime, which the reference keeps private): for
 * checkpoint tooling and tests. */
B2G_API int b2g_bodies_sleep_time_read(b2g_batch* b, int32_t world, int32_t first, int32_t n, float* out);
/* All body states of all worlds as packed arrays (device order = world, then creation order).
 * Any pointer may be NULL. */
B2G_API int b2g_batch_read_states(b2g_batch* b, float* xf4, float* v3, int64_t cap_bodies,
                                  int64_t* n_bodies);
B2G_API int b2g_fixtures_read(b2g_batch* b, int32_t world, int32_t first, int32_t n,
                              b2g_fixture* out);
B2G_API int b2g_joints_read(b2g_batch* b, int32_t world, int32_t first, int32_t n, b2g_joint* out);
/* b2World::GetContactList / b2Contact::GetManifold / IsTouching, b2_world.h:187-191,
 * b2_contact.h:71-143. Contacts are listed in the engine's canonical order. */
B2G_API int b2g_contacts_read(b2g_batch* b, int32_t world, b2g_contact* out, int32_t cap,
                              int32_t* n);
/* b2ContactListener callbacks of the last step, as a batch (see b2g_event): the callbacks the
 * reference makes inside one Step - Begin / End / PreSolve from b2Contact::Update
 * (src/dynamics/b2_contact.cpp:197-209), PostSolve from b2Island::Report
 * (src/dynamics/b2_island.cpp:621-647), End for the touching contacts the broadphase drops
 * (src/dynamics/b2_contact_manager.cpp:48-61) - grouped per world and sorted by kind, then
 * fixture pair. enable != 0 turns event recording on for the batch (off by default; recording
 * costs device time). Events are kept until drained or until the next step begins.
 * b2g_events_drain takes up to `cap` events of the whole batch; b2g_events_drain_world takes
 * only world `world`'s (the others stay for their own drains). */
B2G_API int b2g_events_enable(b2g_batch* b, int32_t enable);
B2G_API int b2g_events_drain(b2g_batch* b, b2g_event* out, int32_t cap, int32_t* n);
B2G_API int b2g_events_drain_world(b2g_batch* b, int32_t world, b2g_event* out, int32_t cap, int32_t* n);
/* b2World::GetProfile, include/box2d/b2_world.h:249 */
B2G_API int b2g_profile_get(b2g_batch* b, b2g_profile* out);
/* The constraint colour and solve-order record of the last step of one world, for replaying the
 * same Gauss-Seidel order on a CPU solver: contact_color[i] for contact i in b2g_contacts_read
 * order (-1 if not solved), joint_color[j] per joint, and the priority keys. */
B2G_API int b2g_solver_order(b2g_batch* b, int32_t world, int32_t* contact_color,
                             uint32_t* contact_priority, int32_t nc, int32_t* joint_color,
                             uint32_t* joint_priority, int32_t nj);

/* ---- world queries (batched; host buffers) ------------------------------------------------- */
/* One ray's closest hit (b2RayCastCallback::ReportFixture returning the fraction). */
typedef struct b2g_ray_hit {
  int32_t fixture;  /* world-local fixture index, -1 when the ray hits nothing */
  float point[2];   /* (1 - fraction) * p1 + fraction * p2 */
  float normal[2];
  float fraction;
} b2g_ray_hit; /* 24 bytes */

/* b2World::QueryAABB (src/dynamics/b2_world.cpp:1193-1207) for n queries at once: query q asks
 * world worlds[q] for the fixtures whose AABB overlaps boxes[4q..4q+3] (lower x, y, upper x, y).
 * counts[q] receives the number of fixtures; fixtures receives them query after query, each
 * query's ascending (world-local indices), at most cap in total; *total is the number found.
 * Returns B2G_E_CAPACITY (counts and total filled, fixtures not) when total > cap. Like the
 * reference, a world of one fixture reports it for every box. */
B2G_API int b2g_query_aabb(b2g_batch* b, const int32_t* worlds, const float* boxes, int32_t n, int32_t* counts,
                           int32_t* fixtures, int64_t cap, int64_t* total);
/* b2World::RayCast (src/dynamics/b2_world.cpp:1228-1238) with a closest-hit callback, for n rays
 * at once: ray q from (rays[4q], rays[4q+1]) to (rays[4q+2], rays[4q+3]) in world worlds[q].
 * Of fixtures hit at the same fraction the lowest index is reported (the reference reports the
 * one its tree visits last). */
B2G_API int b2g_raycast_closest(b2g_batch* b, const int32_t* worlds, const float* rays, int32_t n, b2g_ray_hit* hits);

/* ---- standalone kernels over caller buffers (device pointers) ------------------------------ */
/* Narrowphase: manifolds for n shape pairs (b2CollidePolygons / b2CollideCircles /
 * b2CollidePolygonAndCircle / b2CollideEdgeAndCircle / b2CollideEdgeAndPolygon,
 * include/box2d/b2_collision.h:225-259). Shapes must be ordered like b2Contact::Create's
 * dispatch (src/dynamics/b2_contact.cpp:46-56): A's type >= B's type, edge-edge unsupported.
 * All pointers are device pointers; xf records are (p.x, p.y, q.s, q.c). */
B2G_API int b2g_collide(const b2g_shape* d_shape_a, const float* d_xf_a, const b2g_shape* d_shape_b,
                        const float* d_xf_b, int32_t n, b2g_manifold* d_out, void* stream);
/* Time of impact of n pairs of swept shapes (b2TimeOfImpact, src/collision/b2_time_of_impact.cpp:
 * 258-490), one output per input, same states and times. All pointers are device pointers. */
B2G_API int b2g_time_of_impact(const b2g_toi_input* d_in, int32_t n, b2g_toi_output* d_out, void* stream);
/* Broadphase: every pair (i < j) of the n AABBs (lo.x, lo.y, hi.x, hi.y) that overlap with the
 * reference's inclusive test (include/box2d/b2_collision.h:270-276), sorted by (i, j), written
 * as i << 32 | j into d_pairs (capacity cap). *n_pairs receives the total (64-bit: dense
 * overlap passes 2^31 pairs from about 65 536 boxes), which may exceed cap (then nothing is
 * written and B2G_E_CAPACITY is returned). A traversal that outgrows its stack also returns
 * B2G_E_CAPACITY.
 * Replaces b2BroadPhase::UpdateAndQuery's pair report (include/box2d/b2_broad_phase.h:252-343). */
B2G_API int b2g_pairs(const float* d_aabbs, int32_t n, uint64_t* d_pairs, int64_t cap,
                      int64_t* n_pairs, void* stream);

/* The same pair search as b2g_pairs, for callers that cannot allocate device memory when they
 * call it: a game or robotics loop that must not call cudaMalloc/cudaFree inside its frame (the
 * calls synchronise the device and can stall for milliseconds), or a plug-in running inside a host
 * application that owns the device's memory budget. No counterpart in the reference (its
 * broadphase runs on the CPU and allocates from its own pools).
 * Its scratch is a fixed 16 MiB array in device memory that every GPU loading the library keeps
 * until the process exits (68 bytes per AABB plus the radix sort's temporary storage, which fits
 * at the maximum); n may be at most B2G_PAIRS_STATIC_MAX (larger n returns B2G_E_CAPACITY without
 * touching anything). All calls share the array: calls that overlap on the GPU (two streams, or
 * two host threads) race and must be serialised by the caller. Like b2g_pairs, a call synchronises
 * `stream` twice before it returns (once to read the pair total, once at the end), so it cannot be
 * recorded into a CUDA graph or called while `stream` is being captured.
 * Same outputs, capacity rule and status codes as b2g_pairs. */
#define B2G_PAIRS_STATIC_MAX 131072
B2G_API int b2g_pairs_static(const float* d_aabbs, int32_t n, uint64_t* d_pairs, int64_t cap,
                             int64_t* n_pairs, void* stream);

/* ---- scenes ------------------------------------------------------------------------------------ */
/* Builds one of the seeded benchmark scenes into `world` through the b2World facade calls
 * (box2d-optimized_gb300/scenes/scenes.h). kind: 0 pyramid(rows=n, density=p0, friction=p1),
 * 1 mixed drop(n bodies), 2 chains over pile(n chains, 20 links, p0 circles),
 * 3 batch world(n bodies), 4 joint zoo(n rigs), 5 slider rigs(n rigs), 6 gear rigs(n rigs), 7 bullets(n lanes), with `seed`. counts[3] = bodies, fixtures, joints. */
#define B2G_SCENE_PYRAMID 0
#define B2G_SCENE_MIXED_DROP 1
#define B2G_SCENE_CHAINS 2
#define B2G_SCENE_BATCH_WORLD 3
#define B2G_SCENE_JOINTS 4      /* rigs of weld, wheel, motor, friction, mouse and pulley joints */
#define B2G_SCENE_SLIDERS 5     /* rigs of distance and prismatic joints (n rigs) */
#define B2G_SCENE_GEARS 6       /* rigs of gear joints (n rigs) */
#define B2G_SCENE_BULLETS 7     /* bullets fired at boxes (n lanes; p0 = 1: kinematic bars in every fourth), for continuous collision */
B2G_API int b2g_scene_build(b2g_batch* b, int32_t world, int32_t kind, uint32_t seed, int32_t n,
                            float p0, float p1, int32_t* counts);
B2G_API int b2g_batch_world_params(uint32_t seed, int32_t* n_bodies, float* gx, float* gy);

/* ---- serving ------------------------------------------------------------------------------------ */
typedef struct b2g_server b2g_server;
typedef struct b2g_request_result {
  int64_t request_id;
  int32_t status;           /* B2G_OK, B2G_E_OUT_OF_MEMORY (rejected), ... */
  int32_t bodies;
  int32_t steps;
  double submit_time_s;     /* host monotonic clock */
  double admit_time_s;
  double finish_time_s;
  float checksum[4];        /* sum of x, y, angle, |v| over the world's bodies at the end */
} b2g_request_result;
/* A continuous-batching server: rollout requests (a seeded scene + K steps) are admitted as
 * slots and device memory free up, packed into one batched Step with every other active
 * world, and retired when their K steps are done. Admitted worlds are built on the host by
 * builder threads (2 by default) while the device steps. */
B2G_API int b2g_server_create(int device, uint64_t budget_bytes, int32_t max_worlds,
                              float dt, int32_t velocity_iterations, int32_t position_iterations,
                              b2g_server** out);
B2G_API int b2g_server_destroy(b2g_server* s);
/* Number of host threads that build admitted worlds (0: the tick builds them itself while the
 * device steps). B2G_E_LOCKED while an admitted world is still to be built or joined. */
B2G_API int b2g_server_set_builders(b2g_server* s, int32_t n);
/* Queue a request: scene B2G_SCENE_BATCH_WORLD with `seed`, `bodies` bodies, `steps` steps. */
B2G_API int b2g_server_submit(b2g_server* s, uint32_t seed, int32_t bodies, int32_t steps,
                              int64_t* out_request_id);
/* Admit what fits, run one batched step of all active worlds, retire finished ones.
 * *active receives the number of active worlds (stepped, or uploaded by this step); *step_ms the
 * step's wall time, launch to completion, host work overlapped with it included. */
B2G_API int b2g_server_tick(b2g_server* s, int32_t* active, double* step_ms);
B2G_API int b2g_server_poll(b2g_server* s, b2g_request_result* out, int32_t cap, int32_t* n);
/* Cancels a queued or running request: it finishes at once with status B2G_E_CANCELLED (its
 * world, if admitted, is retired; the other requests are unaffected). B2G_E_INVALID_ARG when the
 * request is unknown or already finished. */
B2G_API int b2g_server_cancel(b2g_server* s, int64_t request_id);
/* The batch the server steps (owned by the server): for reading its profile (b2g_profile_get),
 * querying served worlds or reading their state between ticks. */
B2G_API int b2g_server_batch(b2g_server* s, b2g_batch** out);
B2G_API int b2g_server_stats(b2g_server* s, int64_t* queued, int64_t* active,
                             int64_t* completed, int64_t* rejected, int64_t* hbm_bytes);

/* ---- misc ---------------------------------------------------------------------------------------- */
B2G_API const char* b2g_status_string(int status);
B2G_API const char* b2g_last_error(void);
B2G_API int b2g_device_count(int32_t* n);

#ifdef __cplusplus
}
#endif

#endif /* B2G_CAPI_H */
