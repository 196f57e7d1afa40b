/* gbtissue.h — C ABI of the GB300 XPBD tissue solver (libgbtissue.so).
 *
 * A drop-in for the reference plugin's LCS_* exports on the plain XPBD path
 * (endoscopic_tissue/native/vendor/src/plugin_api.cpp), with the same names, argument meaning,
 * struct layouts and status bands.  Plain pointers and sizes only; host arrays are copied in
 * and out during each call and the caller keeps ownership (V/physics.cu:246-253; "V/" is
 * endoscopic_tissue/native/vendor/cuda/).  One process-global session; not thread safe.
 *
 * Status: 0 ok; -(cudaError_t); -1000..-1005 solver (xpbd_solver.h:25-33); -2000..-2004 physics
 * init (V/physics.cu:219-228); -3000..-3002 cut init (V/cut.cu:1109-1206);
 * LCS_ERR_UNSUPPORTED (-4001): a switch of the reference's unified contact/grasp solver that this
 * library does not provide (contact model 2, grasp capture on model 0, surface-contact entry
 * points); LCS_ERR_DEVICE_TIMEOUT (-4002): a device barrier exceeded its spin budget and the frame
 * was abandoned.
 */
#ifndef GBTISSUE_H
#define GBTISSUE_H

#ifdef __cplusplus
extern "C" {
#endif

#define LCS_API __attribute__((visibility("default")))

#define XPBD_ERR_NOT_READY (-1000)
#define XPBD_ERR_NO_FRAME (-1001)
#define XPBD_ERR_BAD_DT (-1002)
#define XPBD_ERR_COLOR_OVERFLOW (-1003)
#define XPBD_ERR_BAD_ARG (-1004)
#define XPBD_ERR_IRREGULAR_REST (-1005)
#define LCS_ERR_UNSUPPORTED (-4001)
#define LCS_ERR_DEVICE_TIMEOUT (-4002)
#define LCS_ERR_SCRATCH_LIMIT (-4003)

/* ReconInitDesc, 40 bytes (V/dc_recon.h ReconInitDesc; Python ReconDesc, native_backend.py:22-25). */
typedef struct { int voxelCount, cornerCount, isectCount, surfaceEdgeCount, triCapacity, dimsX, dimsY, dimsZ; float L; int qefIters; } ReconInitDescAbi;
/* PhysicsInitDesc, 52 bytes (V/physics.h:18-31). */
typedef struct { int cornerCount, bendPairCount; float ks, cs, kb, cb, hInit, hMax; int maxSubsteps; float alpha, youngE, poisson, strainDamping; } PhysicsInitDesc;
/* CutInitDesc, 60 bytes (V/cut.h:15-27). */
typedef struct { int voxelCount, cornerCount, gridEdgeCount, isectCount, triCapacity, dimsX, dimsY, dimsZ; float voxelL, originX, originY, originZ; int cutPointCapacity; float cutFPInterp, tearStretchRatio; } CutInitDesc;
/* CutToolDesc, 116 bytes (V/cut.h:29-38): swept blade T1=(Sprev,Eprev,E), T2=(Sprev,E,S). */
typedef struct { float t1v0[3], t1v1[3], t1v2[3], t2v0[3], t2v1[3], t2v2[3], ncut[3]; float d; int valid; float aabbMin[3], aabbMax[3]; } CutToolDesc;
/* XpbdGraspParams, 60 bytes (V/xpbd/xpbd_solver.h:250-290). */
typedef struct { float graspThreshold, releaseThreshold, jawGapClosed, coreEllipseFrac, mu, contactAlpha, contactSkin, ccdVelThresh, ccdMaxDisp, ccdOmega, omegaGrasp, coreAlpha, coreBreakForce, graspMaxDisp; int nExemptRings; } GraspParamsAbi;
/* IsectGpu record, 40 bytes (V/common.cuh:23-32). */
typedef struct { float position[3], normal[3]; int a, b; float t; int insideA; } IsectAbi;

/* ---- initialisation (plugin_api.cpp:70-79, 105-115, 138-142) ---------------------------------- */
/* LCS_Init: corner lattice (cornerPos float[3N]) and surface crossings; the dual-contouring buffers
 * (voxelCorner, offsets, counts, surfaceEdges) are accepted and not used.  Replaces recon_init. */
LCS_API int LCS_Init(const ReconInitDescAbi* desc, const float* cornerPos, const int* voxelCorner, const int* voxelIsectOffset,
                     const int* voxelIsectCount, const void* isect, const void* surfaceEdges);
/* LCS_InitPhysics: physics_init + xpbd_bind + xpbd_build_tets (V/physics.cu:214-315). */
LCS_API int LCS_InitPhysics(const PhysicsInitDesc* desc, const float* mass, const int* pinned, const int* active, const float* extForce,
                            const int* nbrIdx, const float* restNbr, const void* bendPairs);
/* LCS_InitCut: cut_init (V/cut.cu:1105-1206); conn4096 is accepted and not used (surface path). */
LCS_API int LCS_InitCut(const CutInitDesc* desc, const void* conn4096, const void* gridEdges, const int* voxelOccupied,
                        const int* cornerInside);
LCS_API int LCS_PhysicsAbiVersion(void);        /* = 52, plugin_api.cpp:102 */
LCS_API int LCS_GraspToolAbiVersion(void);      /* = 92, plugin_api.cpp:197 */
LCS_API int LCS_ContactModelVersion(void);      /* = 28, plugin_api.cpp:225 */

/* ---- per-frame control (plugin_api.cpp:103, 125-166, 145-155, 198-201, 210-214, 263) ---------- */
LCS_API int LCS_SetGravity(float gx, float gy, float gz);           /* physics_set_gravity */
/* physics_step: N substeps + ribbon ticks, then the particle frames (plugin_api.cpp:125-134); a tick
 * that emitted cut points before the last substep is followed by fresh frames (V/physics.cu:368-379) */
LCS_API int LCS_Step(float dt);
LCS_API int LCS_Finalize(void);            /* particle frames from the post-sever lattice (plugin_api.cpp:157-165); no surface rebuild */
LCS_API void LCS_SetTool(const CutToolDesc* tool);                   /* cut_set_tool */
LCS_API int LCS_DetectCut(void);                                     /* cut_detect: swept quad + sever */
LCS_API void LCS_SetPressureCutMode(int enabled);                    /* pressure mode: detection off here */
LCS_API int LCS_SetGraspTool(const void* xpbdToolState);             /* xpbd_set_tool; capture -> -4001 */
LCS_API void LCS_SetGraspParams(const GraspParamsAbi* params);       /* xpbd_set_grasp_params */
/* xpbd_set_contact_model: 0 capsule/jaw-slab CCD gate; 1 tool SDFs (shaft capsule, two jaw boxes)
 * with swept contact and Coulomb friction on lattice nodes (no reconstructed surface); 2 -> -4001. */
LCS_API int LCS_SetContactModel(int enabled, float muS, float muD, float thickness, float radius);
/* xpbd_set_tissue_guard: passes > 0 arms the guarded tet form, `passes` tensile sweeps and the
 * feasibility chain (minimum relative volume `minimum`); `inside`/`capture` concern grasp capture. */
LCS_API int LCS_SetTissueGuard(float minimum, int passes, int count, const int* inside, int capture);
LCS_API int LCS_SetTissueMaterial(float tensileStrength, float bulkDampingSeconds);

/* ---- dual-contouring surface (plugin_api.cpp:84-100; recon_get_counts / recon_get_surface /
 * recon_get_surface_aux, V/dc_recon.cu:625-671).  Rebuilt from the live lattice at LCS_Init and in
 * every LCS_Finalize.  A non-indexed triangle soup: vertexCount == indexCount == 3 x triangles
 * (at most 3 x triCapacity), triangles in surface-edge order; outIdx[i] = i.  Aux = rest anchor xyz
 * + wall flag (0 for the skin). ------------------------------------------------------------------ */
LCS_API int LCS_GetSurfaceCounts(int* vertexCount, int* indexCount);
LCS_API int LCS_GetSurface(float* outPos3, float* outNrm3, int* outIdx);
LCS_API int LCS_GetSurfaceAux(float* outAux4);
/* recon_tri (V/dc_recon.cu:693): the voxel id of every soup vertex, i.e. the indexed form of the
 * surface (vertex v = voxel v's feature point). */
LCS_API int GBT_GetSurfaceTriangles(int* out3T);

/* ---- readback (plugin_api.cpp:38, 170-177) ----------------------------------------------------- */
LCS_API int LCS_GetCornerPos(float* out3N);
LCS_API int LCS_GetNbrIdx(int* out6N);
LCS_API int LCS_GetTopologyRevision(unsigned* revision);
LCS_API int LCS_GetCutEdgeFractions(float* out6N);
LCS_API int LCS_GetCutDebug(unsigned* out18, float* alphaOut);      /* slots 15 (tears) and 16 (cut points) */

/* ---- profiling and shutdown (plugin_api.cpp:21-22, 236-242) ------------------------------------ */
LCS_API void LCS_ProfileEnable(int enabled);
LCS_API int LCS_ProfileRead(int steps, float* ms3);                  /* ms3[0] = device ms of the first `steps` frames */
LCS_API void LCS_ProfileSections(int enabled);                       /* plugin_api.cpp:25 */
LCS_API int LCS_ProfileSectionsRead(char* text, int capacity);       /* plugin_api.cpp:26: "name=ms count=n" lines */
LCS_API void LCS_Shutdown(void);

/* ---- the reference's unified contact/grasp/scissors solver (plugin_api.cpp:30-58, 202-226,
 * 245-261): not provided.  Exported so the reference adapter (native_backend.py:229-263) binds
 * unchanged; the record-size checks answer the reference's layouts, every other call returns
 * LCS_ERR_UNSUPPORTED (-4001) and leaves the session as it was. ------------------------------------ */
LCS_API int LCS_PressureBladeAbiVersion(void);     /* = 52, XpbdBladeState (plugin_api.cpp:259) */
LCS_API int LCS_ScissorsAbiVersion(void);          /* = 244, XpbdScissorsState (plugin_api.cpp:253) */
LCS_API int LCS_ScissorsResultAbiVersion(void);    /* = 124, XpbdScissorsResult (plugin_api.cpp:254) */
LCS_API int LCS_SetPressureBlade(const void* bladeState);                              /* plugin_api.cpp:260 */
LCS_API int LCS_GetPressureBlade(float* values);                                       /* plugin_api.cpp:261 */
LCS_API int LCS_SetScissors(const void* scissorsState);                                /* plugin_api.cpp:255 */
LCS_API int LCS_GetScissors(void* scissorsResult);                                     /* plugin_api.cpp:256 */
LCS_API int LCS_GetScissorsLoads(float* values);                                       /* plugin_api.cpp:257 */
LCS_API int LCS_SetScissorsWrist(float front, float length, float radius);             /* plugin_api.cpp:258 */
LCS_API int LCS_SetJawGeometry(const float* bounds);                                   /* plugin_api.cpp:224 */
LCS_API int LCS_SetKnifeGeometry(int enabled, const float* boxes);                     /* plugin_api.cpp:35 */
LCS_API int LCS_KnifeBodyDepth(float* depth);                                          /* plugin_api.cpp:36 */
LCS_API int LCS_RefineContactSurface(int passes);                                      /* plugin_api.cpp:45 */
LCS_API int LCS_SurfaceDepth(float* depth);                                            /* plugin_api.cpp:32 */
LCS_API int LCS_SetGraspPatch(float sigma, float compliance, float damping);           /* plugin_api.cpp:216 */
LCS_API int LCS_SetToolDynamics(float mass, float stiffness, float damping, float maxTravel);   /* plugin_api.cpp:219 */
LCS_API int LCS_SetJawDynamics(float mass, float stiffness, float damping, float speed);       /* plugin_api.cpp:221 */
LCS_API int LCS_SetInstrumentControl(int guided);                                      /* plugin_api.cpp:218 */
LCS_API int LCS_GetGraspCoreFlags(int count, int* flags);                              /* plugin_api.cpp:226 */
LCS_API int LCS_GetSolvedTool(float* hinge, float* error, int* live);                  /* plugin_api.cpp:220 */
LCS_API int LCS_GetSolvedJaw(float* gap);                                              /* plugin_api.cpp:222 */
LCS_API int LCS_GetContactReaction(float* force, int* contacts);                       /* plugin_api.cpp:202 */
LCS_API int LCS_GetJawLoad(float* load);                                               /* plugin_api.cpp:30 */
LCS_API int LCS_GetMaterialQuality(float* quality);                                    /* plugin_api.cpp:207 */

/* ---- module diagnostics without an LCS_ export in the reference -------------------------------- */
LCS_API int LCS_TetCount(void);                  /* xpbd_tet_count (xpbd_solver.h:202) */
LCS_API int LCS_TetColorCount(void);             /* xpbd_tet_color_count (xpbd_solver.h:203) */
LCS_API int LCS_EdgeColorCount(void);            /* xpbd_color_count (xpbd_solver.h:177) */
LCS_API int LCS_EdgeCount(void);                 /* xpbd_get_edge_count (xpbd_solver.h:183) */
LCS_API int LCS_GetTetIds(int* out4T);           /* xpbd_readback_tet_ids (xpbd_solver.h:208): storage order */
LCS_API int LCS_GetVelocities(float* out3N);     /* xpbd_get_velocities (xpbd_solver.h:174) */
/* physics_particle_rot (V/physics.h:66, V/physics.cu:414): the current particle frames, 9 floats per
 * node (rows of R, RotGpu V/cut.cuh:67).  GBT_GetParticleRot copies them to the host; the device
 * pointer of GBT_ParticleRotDevice stays valid until the next LCS_Step / LCS_Finalize (the frames
 * alternate between two buffers). */
LCS_API int GBT_GetParticleRot(float* out9N);
LCS_API int GBT_ComputeParticleFrames(void);   /* physics_compute_rotations (V/physics.cu:399-411): one frame pass, no surface */
LCS_API void* GBT_ParticleRotDevice(void);

/* ---- extensions (no counterpart in the reference ABI) ------------------------------------------ */
/* Per-tet material: mu*V and kappa*V of every tet in storage order (the order of LCS_GetTetIds);
 * replaces the uniform bake from (E, nu).  The frame compliances become 1/(h^2 * value). */
LCS_API int LCS_SetTetStiffness(int count, const float* muV, const float* kappaV);
LCS_API int LCS_GetTetStiffness(float* muV, float* kappaV); /* the current mu*V, kappa*V, storage order */
LCS_API int LCS_GetTetColors(int* outT);         /* greedy colour of each tet, storage order */
LCS_API int LCS_GetEdgeColors(int* out6N);       /* colour of each lattice edge at its owner slot, else -1 */
LCS_API int LCS_GetBendPairs(void* out);         /* the live 32-byte bend records */
LCS_API int LCS_GetVoxelCutMask(unsigned* outV); /* cumulative 12-bit cut mask per voxel */
/* Cut topology of the live mesh, an unstructured tet mesh built on the device from the current
 * topology (no counterpart in the reference, whose cut severs links, V/cut.cu:719-746, and keeps the
 * bind-time colouring, xpbd_solver.cu:1738-1780).  Live tets are those the liveness rule keeps
 * (xpbd_solver.cu:429-466: crossed tets are removed), in emission order (corner-0 node, then Kuhn
 * type).  Around every node the live tets are grouped by shared faces through the node; group
 * j >= 1 of node v becomes vertex N + base(v) + j - 1 (base: exclusive prefix sum of groups - 1
 * over nodes).  Colours: the reference's greedy first-fit colouring re-run in emission order over
 * those vertices (with nothing cut, the bind-time colouring).
 * GBT_CutTopologyBuild computes it and writes counts4 = {live tets L, duplicated vertices D,
 * colours, relaxation sweeps of the colouring}; when no link has been severed since the previous
 * build of the same session (and no LCS_InitCut or GBT_SetState came between), that product stands
 * and the sweeps are 0.  GBT_GetCutTopology copies tetNodes4L[4L] (vertex
 * ids), tetSourceL[L] (storage index, the order of LCS_GetTetIds), tetColourL[L] and dupParentD[D]
 * (the lattice node of vertex N + j).  -1003 (XPBD_ERR_COLOR_OVERFLOW): more than 128 colours. */
LCS_API int GBT_CutTopologyBuild(int* counts4);
LCS_API int GBT_GetCutTopology(int* tetNodes4L, int* tetSourceL, int* tetColourL, int* dupParentD);
LCS_API int GBT_GetActive(int* outN);           /* physics_active (V/physics.h:69): the live active flags */
/* Restore of the state one LCS_Step hands to the next (no LCS_ export in the reference, which keeps
 * it behind physics_vel / physics_nbr_idx / physics_bend_pairs / physics_active / physics_particle_rot,
 * V/physics.h:66-72, recon_corner_pos, V/dc_recon.h:68, and its cut module's mask, fractions and
 * revision): positions and velocities 3N floats, the neighbour table 6N ints (each slot its lattice
 * neighbour or -1), the 32-byte bend records (only alive flags may differ from the session's), active
 * flags N ints (0/1), voxel cut mask V (12 bits), first-cut edge fractions 6N, particle frames 9N,
 * and the topology revision when setRevision != 0.  Null keeps a table.  A checkpoint is the getters'
 * output; the replay tests load the reference build's state.  Invalid tables: -1004, nothing written. */
LCS_API int GBT_SetState(const float* pos3N, const float* vel3N, const int* nbr6N, const void* bendPairs, const int* active,
                         const unsigned* cutMaskV, const float* edgeCutT6N, const float* rot9N, int setRevision, unsigned revision);
/* Debug builds (libgbtissue_debug.so, compiled with GBT_DEBUG_BOUNDS; the stand-in for a memory
 * checker): every element gather index (edge ends, bend nodes, tet nodes, neighbour-table owner
 * slots) is checked against the nodes the kernel serves; a violation is counted, its index and site
 * (1 edge, 2 bend, 3 tet, 4 edge owner slot, 5 tet owner slot) recorded and the access redirected in
 * range.  out3 = {violations, first index, first site}, cleared by the read.  Release builds:
 * LCS_ERR_UNSUPPORTED. */
LCS_API int GBT_DebugBoundsRead(unsigned* out3);
LCS_API int GBT_BatchDebugBoundsRead(unsigned* out3);
LCS_API int LCS_SetLaunchMode(int mode);         /* 0 automatic, 1 whole-GPU cooperative grid, 2 one CTA, 3 one thread-block cluster (plain frames) */
/* Failure-detection test mode of the grid barrier: every barrier awaits `extraArrivals` arrivals that
 * never come and gives up after `budgetSeconds` (normal budget 2 s); LCS_Step then returns -4002 and
 * the context stays usable.  (0, 2.0) restores normal operation. */
LCS_API int LCS_SetBarrierTest(int extraArrivals, float budgetSeconds);
/* Diagnostics of the whole-GPU frame (no counterpart in the reference).  GBT_FrameBarriers: the grid
 * barriers the last LCS_Step frame executed when it ran on the whole-GPU grid (-1000 otherwise); each
 * closes one phase.  GBT_GridBarrierFloor: microseconds per barrier of `barriers` (1..1e6) back-to-back
 * barriers on the same grid with no work between them, the latency floor of a phase. */
LCS_API int GBT_FrameBarriers(unsigned* barriers);
LCS_API int GBT_GridBarrierFloor(int barriers, float* usPerBarrier);

/* ---- batched instances (no counterpart in the reference, which has one session per process) ----
 * Many independent tissue meshes, each with the topology its own plain session would build, are
 * packed into one table and advanced together, one persistent launch per frame.  Instance inputs are
 * the LCS_InitPhysics arrays of one lattice; tetMuV/tetKappaV (storage order, may be null) replace the
 * (E, nu) bake like LCS_SetTetStiffness.  Instruments: contact model 0 capsules, one XpbdToolState
 * (92 B) per instance per frame.  Every instance shares the lattice spacing and parameters below. */
typedef struct { int dimsX, dimsY, dimsZ; const float* cornerPos; const float* mass; const int* pinned; const int* active;
                 const int* nbrIdx; const float* restNbr; const void* bendPairs; int bendPairCount;
                 const float* tetMuV; const float* tetKappaV; float stiffnessScale; } GbtInstanceDesc;
/* stiffnessScale > 0 multiplies both per-tet stiffnesses (after any override), in FP32: an instance of
 * Young's modulus E' is stiffnessScale = E'/E of the bake. */
typedef struct { int substeps; float ks, cs, kb, cb, alpha, youngE, poisson, strainDamping; } GbtBatchParams;
LCS_API int GBT_BatchInit(int count, const GbtInstanceDesc* instances, const GbtBatchParams* params);
LCS_API int GBT_BatchSetGravity(float gx, float gy, float gz);
LCS_API void GBT_BatchSetGraspParams(const GraspParamsAbi* params);
LCS_API int GBT_BatchSetTools(const void* xpbdToolStates);            /* count x 92 B: the next frame's instruments */
LCS_API int GBT_BatchStep(float dt);                                   /* one frame of every instance */
/* `steps` frames; tools = [steps][count] XpbdToolState or null; useGraph: replay the launches from a
 * CUDA graph captured on first use (recaptured when steps, launch shape or dt change). */
LCS_API int GBT_BatchStepMany(float dt, int steps, const void* tools, int useGraph);
LCS_API int GBT_BatchGetPositions(float* out3N);                      /* all nodes, instance after instance */
LCS_API int GBT_BatchNodeRange(int instance, int* base, int* count);
LCS_API int GBT_BatchInfo(int* counts8);                               /* instances, nodes, edges, tets, edge colours, tet colours, mode, threads */
/* Launch shape: mode 0 lockstep grid (threads 256), 1 one CTA per instance (threads 256 | 512),
 * 2 one thread-block cluster per instance list with positions in distributed shared memory
 * (`threads` = CTAs per cluster: 2 | 4 | 8; -4001 when the largest instance does not fit). */
LCS_API int GBT_BatchSetLaunch(int mode, int threads);
/* Instance packing of the shapes that give an instance to one CTA or cluster (modes 1, 2): 0 longest
 * processing time first on tet counts (the default), 1 the same on tets + edges + nodes, 2 instances
 * in decreasing size dealt round-robin in serpentine order.  Identical results in every packing. */
LCS_API int GBT_BatchSetPacking(int packing);
LCS_API int GBT_BatchPacking(void);
/* Times every configuration for trialSteps frames from the current state (put back afterwards) and
 * keeps the fastest: the lockstep grid on each element-table form, one CTA per instance at 256 and
 * 512 threads and clusters of 2, 4 and 8 CTAs, each with the three packings.  msPerFrame6 gets the
 * best ms per frame of each shape {0/256, 1/256, 1/512, 2/2, 2/4, 2/8} (-1: not usable for this
 * batch).  GBT_BatchAutotuneTable copies up to `capacity` trials -- (mode, threads, packing,
 * implicit element tables) in shape4, ms per frame in ms (-1: not usable) -- and returns how many
 * the last autotune ran. */
LCS_API int GBT_BatchAutotune(float dt, int trialSteps, int* modeOut, int* threadsOut, float* msPerFrame6);
LCS_API int GBT_BatchAutotuneTable(int capacity, int* shape4, float* ms);
/* Element tables of the frame kernels: 1 implicit lattice codes -- 4 bytes per tet and per edge (plus
 * the edge rest length), nodes and compliances derived from the instance's lattice strides and
 * Kuhn type -- used by default when every instance qualifies (instances of < 32,768 nodes, fewer
 * than 8,192 instances, one stiffness per instance and Kuhn type, ks > 0); 0 the explicit tables
 * (node ids, flags and compliance per element).  Identical results; returns -4001 when 1 is asked
 * of a batch that does not qualify.  GBT_BatchElementTables: the form in use (1 / 0). */
LCS_API int GBT_BatchSetElementTables(int implicitCodes);
LCS_API int GBT_BatchElementTables(void);
LCS_API void GBT_BatchProfileEnable(int enabled);
LCS_API int GBT_BatchProfileRead(float* msTotal);                      /* device ms of the profiled step calls */
LCS_API void GBT_BatchShutdown(void);

/* ---- differentiable rollout (no counterpart in the reference, whose solver is not differentiable)
 * Runs the plain substep (predict, lattice edges, unguarded Neo-Hookean tets, capsule contact of
 * the shaft, velocity update) on the LCS session's mesh and returns adjoints of the final node
 * positions' loss.  Every array argument of GBT_DiffForward / GBT_DiffBackward is DEVICE memory on
 * the session's device (a torch CUDA tensor's data pointer); sizes: N nodes, T tets (storage order,
 * as LCS_SetTetStiffness), F frames.  Sessions with bending, perpendicular damping, edge-only
 * fallback, an active blade or contact model != 0 return LCS_ERR_UNSUPPORTED.                    */
/* Take the session's current state as the rollout origin and its per-tet stiffness as the bake
 * that log-compliances scale: (mu V, kappa V) * 1 / (exp(theta) * scaleModulus) (scaleModulus =
 * the bake's Young's modulus in Pa makes exp(theta) a Young's compliance in 1/Pa).  Checkpoints
 * are kept every checkpointEvery substeps; buffers are sized for up to maxFrames frames. */
LCS_API int GBT_DiffBegin(float scaleModulus, int checkpointEvery, int maxFrames);
/* F frames from the origin.  logCompliance float[T]; capsulePath float[(F + 1) * 6] = end points
 * (a, b) of the capsule per command, frame f moving from command f to f + 1 (NULL: no instrument);
 * finalPos float[3N] or NULL.  The session is left at the final state. */
LCS_API int GBT_DiffForward(float dt, int frames, const float* logCompliance, const float* capsulePath, float capsuleRadius,
                            float* finalPos);
/* Adjoint of the last forward.  gradPos float[3N] in; out: gradLogCompliance float[T];
 * gradCapsulePath float[(F + 1) * 6] or NULL; gradRestLength float[6N] by directed slot 6p + s of
 * the edge's owner (rest length of each lattice edge) or NULL; gradRestInverse float[9T] (each
 * tet's rest inverse Dm^-1, row major, storage order) or NULL; gradOrigin float[6N] (3N position
 * then 3N velocity adjoints of the origin state) or NULL. */
LCS_API int GBT_DiffBackward(const float* gradPos, float* gradLogCompliance, float* gradCapsulePath, float* gradRestLength,
                             float* gradRestInverse, float* gradOrigin);
LCS_API int GBT_DiffInfo(int* out4);   /* grid launch (1) or one CTA (0), CTAs, checkpoint interval, max frames */
LCS_API void GBT_DiffEnd(void);

/* LCS_StepNoAlloc has no counterpart in the reference.  It advances the session by one frame
 * exactly as LCS_Step does, in the launch shape LCS_Step would pick (automatic mode: the shape its
 * timed trials kept, or before them one CTA where the nodes fit its shared memory, else the whole
 * GPU; it runs no trials itself), for hosts that cannot let a plugin allocate GPU memory while they
 * run (engines that own every device allocation through their own pool or budget, and real-time
 * loops where an allocation, which may synchronise the device, would stall a frame).  It calls no
 * cudaMalloc, cudaFree or other allocating routine: the frame's scratch (barrier counter, status,
 * liveness record, per-tet compliances) is a fixed 4 MiB + 256 B array inside the library, which
 * every GPU that loads the library holds until the process exits.  Limit: meshes of at most
 * 524,288 tets; larger ones return LCS_ERR_SCRATCH_LIMIT (-4003) without stepping.  The first call
 * after each LCS_Init looks up that array's device address on the current device, so make it before
 * any stream capture.  All calls in one process share the array; the library is not thread safe,
 * and two host threads stepping at once would race on it.  Frames stepped here are not recorded by
 * LCS_ProfileEnable.  The inputs and outputs are the session's buffers set up by
 * LCS_Init/LCS_InitPhysics/LCS_InitCut; the status is LCS_Step's. */
LCS_API int LCS_StepNoAlloc(float dt);

#ifdef __cplusplus
}
#endif
#endif
