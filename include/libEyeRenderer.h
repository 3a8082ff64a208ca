/*
 * libEyeRenderer3 — headless compound-eye renderer for one GB300 GPU.
 *
 * Drop-in C ABI for the reference's libEyeRenderer3
 * (BrainsOnBoard/compound-ray, libEyeRenderer3/libEyeRenderer.h:16-67).
 * Every reference entry point keeps its name, signature and meaning; each
 * declaration below cites the reference declaration it replaces.  No window
 * is opened when the library loads.  Errors never throw across the ABI:
 * they set a message readable with crGetLastError() and the function returns
 * its sentinel (the reference's own sentinels where it has one).
 *
 * The entry points prefixed "cr" have no counterpart in the reference; they
 * expose the per-ommatidium fp32 colours, batched pose trajectories and the
 * test/diagnostic views the parity tests need.
 *
 * Not thread-safe: one process-wide renderer, as in the reference.
 */
#ifndef LIB_EYE_RENDERER_3_H
#define LIB_EYE_RENDERER_3_H

#include <cstddef>
#include <cstdint>
#include <vector_types.h>

/* Same layout as the reference's OmmatidiumPacket (libEyeRenderer.h:8-14). */
struct OmmatidiumPacket {
  float posX, posY, posZ;
  float dirX, dirY, dirZ;
  float acceptanceAngle;
  float focalpointOffset;
};

extern "C" {
/* ---- Configuration (libEyeRenderer.h:18-26) ---------------------------- */
void setVerbosity(bool v);                /* libEyeRenderer.h:19 */
void loadGlTFscene(const char* filepath); /* libEyeRenderer.h:20; replaces any scene loaded before */
void stop(void);                          /* libEyeRenderer.h:21; frees every GPU resource */
void setRenderSize(int w, int h);         /* libEyeRenderer.h:22 */
double renderFrame(void);                 /* libEyeRenderer.h:23; ms, -1.0 on error */
void displayFrame(void);                  /* libEyeRenderer.h:24; no display here: no-op */
void saveFrameAs(char* ppmFilename);      /* libEyeRenderer.h:25; binary PPM, rows flipped */
unsigned char* getFramePointer(void);     /* libEyeRenderer.h:26; h*w*4 bytes owned by the library */

/* ---- Camera control (libEyeRenderer.h:28-49) --------------------------- */
size_t getCameraCount(void);              /* :29 */
void nextCamera(void);                    /* :30 */
void previousCamera(void);                /* :31 */
size_t getCurrentCameraIndex(void);       /* :32 */
const char* getCurrentCameraName(void);   /* :33 */
void gotoCamera(int index);               /* :34 */
bool gotoCameraByName(char* name);        /* :35 */
void setCameraPosition(float x, float y, float z);      /* :36 */
void getCameraPosition(float& x, float& y, float& z);   /* :37 */
void setCameraLocalSpace(float lxx, float lxy, float lxz, float lyx, float lyy, float lyz, float lzx, float lzy,
                         float lzz);                    /* :39-41 */
void rotateCameraAround(float angle, float axisX, float axisY, float axisZ);        /* :42 */
void rotateCameraLocallyAround(float angle, float axisX, float axisY, float axisZ); /* :43 */
void translateCamera(float x, float y, float z);                                    /* :44 */
void translateCameraLocally(float x, float y, float z);                             /* :45 */
void resetCameraPose(void);                                                         /* :47 */
void setCameraPose(float posX, float posY, float posZ, float rotX, float rotY, float rotZ); /* :49 */

/* ---- Compound-eye control (libEyeRenderer.h:53-61) --------------------- */
bool isCompoundEyeActive(void);                          /* :53 */
void setCurrentEyeSamplesPerOmmatidium(int s);           /* :54; resets the random streams */
int getCurrentEyeSamplesPerOmmatidium(void);             /* :55; -1 if not compound */
void changeCurrentEyeSamplesPerOmmatidiumBy(int s);      /* :56 */
size_t getCurrentEyeOmmatidialCount(void);               /* :57; 0 if not compound */
void setOmmatidia(OmmatidiumPacket* omms, size_t count); /* :59 */
const char* getCurrentEyeDataPath(void);                 /* :60; "" if not compound */
void setCurrentEyeShaderName(char* name);                /* :61 */

/* ---- Scene queries (libEyeRenderer.h:64-66) ---------------------------- */
bool isInsideHitGeometry(float x, float y, float z, char* name); /* :64 */
float3 getGeometryMaxBounds(char* name);                        /* :65 */
float3 getGeometryMinBounds(char* name);                        /* :66 */

/* ---- Additions (no counterpart in the reference) ----------------------- */

/* isInsideHitGeometry for n points at once on the GPU: points n x 3 floats
 * (world space), inside n bytes (1 = inside the hitbox mesh `name`), the
 * same parity ray cast and answers as isInsideHitGeometry point by point
 * (sutil/hitscanprocessing.cpp:20-83).  0 on success, -1 for an unknown
 * hitbox or a CUDA error. */
int crInsideHitGeometryBatch(const float* points, size_t n, const char* name, unsigned char* inside);

/* Copies the last error message (NUL-terminated, truncated to len) and
 * returns its full length; 0 when no error is pending.  Reading clears it. */
int crGetLastError(char* buf, size_t len);

/* Per-ommatidium fp32 RGB of the last compound render of the current eye:
 * N x 3 floats, each the sum over samples of colour/spp before the gamma
 * and 8-bit conversion of getFramePointer (shaders.cu:341-347).  0 on success. */
int getOmmatidialColoursF32(float* out);

/* Renders `count` poses of the current compound eye as `count` consecutive
 * frames (the random streams advance one frame per pose, exactly as `count`
 * calls of renderFrame would) in batched launches.
 * poses: count x 12 floats = position xyz, local x axis, local y axis,
 *        local z axis (host memory).  out: count x N x 3 floats (host).
 * Leaves the camera pose unchanged.  Returns 0 on success. */
int crRenderPoses(const float* poses, size_t count, float* out);

/* As crRenderPoses with device pointers: d_poses = count x 16 floats
 * (position, x, y, z axes as float4 each, w ignored), d_out = count x N x 3.
 * Runs asynchronously on the library stream (see crSetStream). */
int crRenderPosesDevice(const float* d_poses, size_t count, float* d_out);

/* No counterpart in the reference.  crRenderPosesDevice for callers that
 * cannot allocate device memory at render time -- e.g. code running while a
 * CUDA stream is being captured into a graph, real-time loops that cannot
 * take cudaMalloc's implicit synchronisation, or hosts whose device memory is
 * owned by another allocator.  The call makes no cudaMalloc or cudaFree: the
 * per-chunk partial sums go to a fixed 16 MiB device array inside the
 * library (held by every GPU that loads it until exit) instead of a
 * library-allocated buffer.  Limits and rules:
 *  - an eye needing more than 4 Mi floats of scratch per pose
 *    (N * ceil(spp/32) * 3 when spp > 32) is rejected with an error;
 *  - the current eye must already have been rendered once through an
 *    allocating entry point with its present ommatidium and sample counts,
 *    so that its device state exists;
 *  - the first call on each device looks up the array's device address; make
 *    that first call before any stream capture;
 *  - every call shares the array: calls that overlap on the GPU race;
 *  - it does not spread the poses of a small eye over extra warps (that
 *    needs a buffer of pre-drawn random numbers) and ignores the near-field
 *    cut radius (the cuts need a buffer too), so small eyes and near-field
 *    scenes render more slowly through it.
 * Results are bit-identical to crRenderPosesDevice's.  0 on success. */
int crRenderPosesDeviceNoAlloc(const float* d_poses, size_t count, float* d_out);

/* Batched rendering of several compound cameras of the scene in ONE
 * persistent launch (work-queue kernel over every eye's warp tasks),
 * recorded once into a CUDA graph and replayed by crBatchLaunch.
 *  cams: nCams camera indices (each a compound eye, each at most once);
 *  d_poses: device, nCams x posesPerCam poses of 16 floats, camera-major;
 *  d_out: device, each camera's posesPerCam x N x 3 floats at float offset
 *         crBatchOutputOffset(handle, i), cameras one after another.
 * Each launch renders every camera's poses as consecutive frames of that
 * camera (its random streams advance exactly as crRenderPosesDevice's
 * would).  The eyes keep the sample counts and ommatidia they had at
 * creation; any later change of the scene or of an eye invalidates the
 * batch (crBatchLaunch then fails).  Returns a handle > 0, or -1. */
int crBatchCreate(const int* cams, size_t nCams, size_t posesPerCam, const float* d_poses, float* d_out);
int crBatchLaunch(int handle);
/* After a launch: per-camera completion time of its last warp task and of
 * the whole batch, in ms from the start of the launch (synchronises). */
int crBatchLatencies(int handle, float* msPerCam, float* totalMs);
size_t crBatchOutputOffset(int handle, size_t camIndex);
int crBatchDestroy(int handle);
/* One-shot batch: crBatchCreate, one launch, a wait for it, crBatchDestroy.
 * Camera i's frames start at float offset 3 * posesPerCam * (the ommatidium
 * counts of cams[0 .. i-1] summed) of d_out.  0 on success, -1 on error. */
int renderBatch(const int* cams, size_t nCams, size_t posesPerCam, const float* d_poses, float* d_out);

/* Diagnostic: renders `count` device poses (layout of crRenderPosesDevice)
 * of the current eye and reports the mean BVH node visits and triangle tests
 * per ray.  Advances the random streams like a render.  0 on success. */
int crMeasureTraversal(const float* d_poses, size_t count, double* nodesPerRay, double* trisPerRay);

/* Autotuner: times every variant of the render kernel on `count` device
 * poses of the current eye (layout of crRenderPosesDevice), keeps the
 * fastest for the rest of the process and reports it (and, if msPerVariant
 * is not null, crGetRenderVariantCount() timings).  The eye's random streams
 * are restored after every trial, so tuning changes no result.  0 on success. */
int crAutotune(const float* d_poses, size_t count, int* bestVariant, float* msPerVariant);
/* No counterpart in the reference.  After the variants, crAutotune times
 * the block size (128, 256, 512 threads), then the samples per warp segment
 * (8, 16, 32), then the near-field cut radius, keeping the fastest of each;
 * a non-zero best radius is refined by trying it divided and multiplied by
 * sqrt(2).  Last it times the BVH widths 4 and 8 (crSetBvhWidth) against the
 * two-wide BVH with its best cut, and keeps the fastest tree.
 * crGetAutotuneTimes copies its timings (ms): variants 0-2, blocks 128 / 256
 * / 512, samples per warp 8 / 16 / 32, cut radius 0, 1/256, 1/128, 1/64,
 * 1/32, 1/16 of the scene extent, BVH width 2 / 4 / 8, and the refinement's
 * radius / sqrt 2 and x sqrt 2 (20 values; the last two 0 when the best
 * radius was 0). */
int crGetAutotuneTimes(float* ms, size_t n);
/* No counterpart in the reference.  Layout of the render kernel: block size
 * in threads (0 = the smallest of 128 / 256 / 512 holding all 32-sample
 * chunk warps of an ommatidium, whose chunk sums then stay in shared memory;
 * else 128) and samples per warp segment (8, 16 or 32; below 32 a warp
 * holds several ommatidia, and the samples are summed in another order:
 * results change within float rounding).  The block size changes no result.
 * Also used by batches created afterwards.  0 on success. */
int crSetRenderLayout(int blockThreads, int samplesPerWarp);
int crGetRenderLayout(int* blockThreads, int* samplesPerWarp);
/* Near-field cut: the radius, as a fraction of the scene's largest vertex
 * coordinate, of the ball around each pose position whose BVH subtrees every
 * ray searches first (0 = off, the default).  A hit found there within the
 * ball is final; other rays continue from the root, so results never depend
 * on it.  crAutotune also picks this radius among 0 and 1/256 .. 1/16.
 * No counterpart in the reference. */
int crSetCutRadius(float fractionOfExtent);
/* Lighting-on shading (shaders.cu:812-880): 1 = the GGX/Smith path with four
 * point lights around the scene's bounding box and shadow rays, from metallic
 * / roughness factors, metallic-roughness and normal textures and vertex
 * normals; 0 = off, the default (the reference's params.lighting is false,
 * libEyeRenderer.cpp:98).  The plain render entry points honour it; batched,
 * learned and adaptive renders refuse to run while it is on.  No counterpart
 * in the reference's API. */
int crSetLighting(int on);
int crGetLighting(void);
/* The loaded scene's lighting-on data: 20 floats per triangle (world vertex
 * normals n0 n1 n2, texture coordinates uv0 uv1 uv2, metallic, roughness,
 * metallic-roughness texture, normal texture, flags 1 = normals 2 = texture
 * coordinates), the four lights' position + intensity (16 floats) and
 * colours (12 floats).  Null pointers are skipped.  0 on success. */
int crGetSceneLighting(float* light, float* lightPos, float* lightCol);
float crGetCutRadius(void);
int crSetRenderVariant(int variant);
int crGetRenderVariant(void);
int crGetRenderVariantCount(void);
/* Candidate search of the spherical projections (spherical_positionwise,
 * _orientationwise, _split_orientationwise and the _ids forms): 0 (default)
 * searches grids of the ommatidia binned by unit vector around each pixel's
 * point, 1 tests every ommatidium as the reference's shaders do
 * (shaders.cu:412-640).  Both give the same image.  No counterpart in the
 * reference. */
int crSetProjectionSearch(int mode);
int crGetProjectionSearch(void);
/* Failure-path knobs, no counterpart in the reference.
 * crSetDeviceMemoryCap: device bytes the library's buffers may hold in
 * total (0: no cap, the default); an allocation past it fails like an
 * out-of-memory cudaMalloc: the call returns its error sentinel and the
 * library stays usable.  crGetDeviceMemoryHeld: the bytes they hold now.
 * crSelfTestBoundedWait: runs the tcgen05 kernels' bounded mbarrier wait on
 * a barrier that nothing arrives on, for `polls` polls; 1 when the wait ran
 * out and reported it through the error word (then cleared), 0 when it did
 * not, -1 on a CUDA error. */
int crSetDeviceMemoryCap(size_t bytes);
size_t crGetDeviceMemoryHeld(void);
int crSelfTestBoundedWait(unsigned int polls);

/* ---- Learned per-ommatidium denoiser ------------------------------------
 * A 4-layer MLP (feature row of 112 -> 128 -> 128 -> 128 -> 3, ReLU) that
 * predicts a correction to an ommatidium's low-sample mean colour from the
 * sample statistics (mean, spread, hit fraction, depth, normal), axis and
 * acceptance angle of the ommatidium and of its 6 nearest ommatidia.  It is
 * trained and run on the GPU with bf16 tensor-core GEMMs accumulating in
 * fp32 and Adam on fp32 master weights.  Its feature renders use their own
 * random streams; the camera's streams are not touched. */
int crDenoiserInit(int seed);                 /* fresh He-initialised weights */
size_t crDenoiserParamCount(void);
void crDenoiserRelease(void);                 /* drops the network (the adaptive render then uses feature means) */
/* Tensor-core path of the networks: 0 = mma.sync (the fused inference
 * kernel is then bit-identical to the layer-by-layer path, and training runs
 * its GEMMs on mma.sync), 1 = tcgen05 with accumulators in TMEM for the
 * fused inference kernel and the training GEMMs (the default).  Set it
 * before crDenoiserTrain / crAllocatorTrain to train on that path.  -1 on a
 * bad kind. */
int crSetDenoiserKernel(int kind);
int crGetDenoiserKernel(void);
/* Renders `count` host poses (12 floats each) of the current eye twice --
 * a featureSpp-sample feature render and a targetSpp-sample plain render --
 * and appends count x N (features, target) rows to the training set. */
int crDenoiserAddTrainingPoses(const float* poses12, size_t count, int featureSpp, int targetSpp);
size_t crDenoiserTrainingRows(void);
/* `steps` Adam steps on shuffled minibatches, the step size decaying from
 * lr by a half cosine to 5% of it over the call; lossHistory: steps floats
 * (mean squared error per step) or null.  The first step runs as plain
 * launches; the rest replay it from a CUDA graph, with the loop's position
 * kept on the device (the host waits only to reshuffle between epochs). */
int crDenoiserTrain(int steps, int batch, float lr, int seed, float* lossHistory);
/* The learned form: featureSpp-sample render + network, count x N x 3
 * (one fused feature + network kernel after the feature render). */
int crDenoiserRenderPosesDevice(const float* d_poses, size_t count, int featureSpp, float* d_out);
int crDenoiserRenderPoses(const float* poses12, size_t count, int featureSpp, float* out);
/* The feature render's rows for host poses: x count*N x 112 bf16 bit
 * patterns, base count*N x 3 (own mean colour); advances the feature
 * streams like a learned render.  And the layer-by-layer prediction of host
 * rows, base + network(x), rows x 3.  Test access, no reference
 * counterpart. */
int crDenoiserFeatureRows(const float* poses12, size_t count, int featureSpp, uint16_t* xBf16, float* base);
int crDenoiserPredictRows(const uint16_t* xBf16, const float* base, size_t rows, float* out);

/* ---- Learned sample allocator and adaptive rendering ---------------------
 * A second network of the denoiser's shape predicts, from the same
 * featureSpp-sample features, how many samples each ommatidium needs:
 * log2(count) / 10 in each output.  Training labels come from a
 * minimum-sample search: every (pose, ommatidium) is rendered `seeds` times
 * with independent streams at 4, 8, ..., 1024 samples, and its label is the
 * first count at which the colour's standard deviation across the renders is
 * below `threshold` in every channel (0 when none is, i.e. more than 1024).
 * No counterpart in the reference. */
int crAllocatorInit(int seed);
/* count <= 256 host poses (12 floats); labelsOut: null or count x N words. */
int crAllocatorAddTrainingPoses(const float* poses12, size_t count, int featureSpp, float threshold, int seeds,
                                uint16_t* labelsOut);
int crAllocatorTrain(int steps, int batch, float lr, int seed, float* lossHistory);
size_t crAllocatorTrainingRows(void);
int crAllocatorSave(const char* path);
int crAllocatorLoad(const char* path);
/* The adaptive learned form of `count` device poses (16 floats each) into
 * d_out (count x N x 3): a featureSpp-sample feature render; the allocator's
 * count c per (pose, ommatidium); where c <= featureSpp the denoised feature
 * estimate (the feature mean when no denoiser is trained); where featureSpp <
 * c <= 1024 an extra c-sample render combined with the feature samples by
 * sample count; where c > 1024 (the predicted variance at 1024 samples is
 * above the threshold) a plain 1024-sample render alone.  An entry's extra
 * samples are the points of a randomly shifted two-dimensional Sobol' net
 * (stratified over its cone; unbiased).  d_level: null,
 * or count x N bytes receiving each entry's bucket (index k = 4 << k samples,
 * 0x88 = 1024-sample fallback, 0xFF = feature render only).  raysTraced:
 * null, or receives the rays of the call.  0 on success. */
int crAdaptiveRenderPosesDevice(const float* d_poses, size_t count, int featureSpp, float* d_out, uint8_t* d_level,
                                double* raysTraced);
/* Error budget of the adaptive render: every predicted count (capped at
 * 2048) is divided by 2^halvings before it is rounded up to a bucket
 * (-4 <= halvings <= 6, fractions allowed; 0, the default, renders each entry
 * to the 1/512 standard deviation of its label; negative values render more
 * samples than predicted, up to 1024).  Each halving raises an
 * extra-sampled entry's expected error by about sqrt(2); from 1 on no entry
 * falls back to the plain 1024-sample render.  Callers pick the largest
 * value that keeps their aggregate error target on validation poses.  No
 * counterpart in the reference. */
int crSetAllocatorHalvings(float halvings);
float crGetAllocatorHalvings(void);
/* No counterpart in the reference.  Shape of the allocation: the count
 * rendered for an entry is 2^(exponent * log2(predicted count) - halvings),
 * exponent in [0.25, 1] (default 1: proportional to the predicted count).
 * The predicted count is the one that brings the entry's standard deviation
 * to 1/512, so it grows with the entry's variance; exponent 1/2 makes the
 * rendered count proportional to the standard deviation instead, which for
 * a given number of rays minimises the aggregate squared error (Neyman
 * allocation).  0 on success. */
int crSetAllocatorExponent(float exponent);
float crGetAllocatorExponent(void);
/* No counterpart in the reference.  Cost term of the allocation: the count
 * is further divided by (cost / 16)^costExponent, cost the entry's mean BVH
 * node visits plus triangle tests per ray in the feature render (at least
 * 1).  costExponent in [0, 1], default 0 (no cost term).  For a fixed
 * render time, rather than a fixed number of rays, the aggregate squared
 * error is smallest with counts in proportion to sigma / sqrt(cost):
 * exponent 1/2 and costExponent 1/2.  With a cost term the allocation
 * depends on how the rays traverse: the near-field cut radius, the BVH
 * builder and its width change the costs, and so which entries get how many
 * samples (no ray's hit changes).  0 on success. */
int crSetAllocatorCostExponent(float costExponent);
float crGetAllocatorCostExponent(void);
/* No counterpart in the reference.  Copies what the last pass of the last
 * crAdaptiveRenderPosesDevice call decided (a call covers its poses in
 * passes of at least 256 poses and up to 2^21 entries): per entry (pose-
 * major, rows = poses of the pass x ommatidia) the allocator's three outputs
 * (prediction: rows x 3 floats; the predicted count is 2^(10 x their mean)),
 * the feature render's traversal cost (cost: rows floats) and the level
 * (level: rows bytes, as crAdaptiveRenderPosesDevice writes it).  Any
 * pointer may be null.  rows must equal the pass's rows.  Any later call
 * that renders features (training, the denoised render) replaces the pass;
 * the call then fails.  0 on success. */
int crAdaptiveLastPass(float* prediction, float* cost, uint8_t* level, size_t rows);
/* No counterpart in the reference.  Ray-refill schedule of the adaptive
 * render: each warp works through a pool of up to 256 samples, traversing in
 * bursts of `steps` BVH steps; between bursts its idle lanes take new samples
 * once at least refillIdle (1..32) of its 32 lanes are idle (32 = whole
 * rounds of 32 rays, no refill).  Defaults 16 and 16.  Results do not depend
 * on it (each entry's samples are summed in a fixed order).  0 on success. */
int crSetAdaptiveSchedule(int refillIdle, int steps);
int crGetAdaptiveSchedule(int* refillIdle, int* steps);
/* No counterpart in the reference.  Occupancy of the adaptive render's kernel
 * on the two-wide BVH: resident 128-thread blocks per SM its register budget
 * is sized for, 5 (96 registers, the default), 6 (80) or 8 (64).  Results do
 * not depend on it.  0 on success. */
int crSetAdaptiveOccupancy(int blocksPerSM);
int crGetAdaptiveOccupancy(void);
/* Test access: `spp` samples per (pose, ommatidium) of host poses, the
 * adaptive render's stratified net draws with one seed, recording every ray (records: count x N x spp, as
 * crRenderFrameRecorded) and the per-entry means (sums: count x N x 3). */
int crAdaptiveRecord(const float* poses12, size_t count, int spp, unsigned long long seed, void* records,
                     float* sums);
/* One forward/backward pass on host rows (x: rows x 112 bf16 bit patterns,
 * base/target: rows x 3): returns the loss (-1 on error) and writes the
 * gradients and the current parameters (crDenoiserParamCount floats each). */
float crDenoiserGradient(const uint16_t* xBf16, const float* base, const float* target, int rows, float* grads,
                         float* params);
/* No counterpart in the reference.  Test access: one Adam step of the
 * training loop's kernel (b1 = 0.9, b2 = 0.999, eps = 1e-8; the step size lr
 * and bias corrections c1 = 1/(1-b1^t), c2 = 1/(1-b2^t) read from a device
 * schedule entry, as in training) on n host parameters: updates w, m, v in
 * place and writes the bf16 bit patterns of the new weights.  0 on success. */
int crDenoiserAdamStep(float* w, const float* g, float* m, float* v, size_t n, float lr, float c1, float c2,
                       uint16_t* wbBits);
/* No counterpart in the reference.  Scales the denoiser's correction by
 * alpha in [0, 1] (its linear output layer is multiplied by alpha; 0 gives
 * the feature render's 8-sample mean): the strength a caller picks on
 * validation poses.  0 on success. */
int crDenoiserScaleOutput(float alpha);
/* Checkpoint of the parameters and Adam moments (binary, with a header). */
int crDenoiserSave(const char* path);
int crDenoiserLoad(const char* path);

/* No counterpart in the reference (whose trees live inside OptiX).  Width
 * of the BVH the closest-hit searches use: 2 (the two-wide BVH, default; the
 * only one with the near-field cut), 4 or 8 (a wide BVH with 8-bit quantised
 * child boxes, collapsed from the two-wide one at the first render that
 * needs it).  Results are identical for every width.  0 on success. */
int crSetBvhWidth(int width);
int crGetBvhWidth(void);
/* No counterpart in the reference.  Test access: the wide BVH of `width`
 * (4 or 8) collapsed on the host from a scene loaded with the host builder
 * and not yet rendered (wbvh.hpp layout, 16 or 24 floats per node), and
 * (trisOut, may be null) the triangles in leaf order, 9 floats each; nodesOut
 * may be null to get the count only. */
int crGetWideBvhHost(int width, float* nodesOut, size_t capFloats, uint32_t* nodeCount, float* trisOut);
/* Wide BVH in use: nodes, depth and mean children per node (0 for width 2). */
int crGetWideBvhStats(uint32_t* nodes, uint32_t* depth, double* meanChildren);

/* BVH builder for scenes loaded afterwards: 0 = host binned SAH (default),
 * 1 = GPU linear BVH (Morton codes, radix sort, Karras hierarchy) built at
 * the first render.  Results are identical either way (the closest hit does
 * not depend on the tree); only speed differs.  0 on success. */
int crSetBvhBuilder(int kind);
int crGetBvhBuilder(void);

/* Makes the library launch on `stream` (a cudaStream_t; null = the library's
 * own stream).  Returns 0 on success. */
int crSetStream(void* stream);

/* Blocks until the library stream is idle; returns 0 or -1 on a CUDA error. */
int crSynchronize(void);

/* Renders one frame of the current compound eye at the current pose and
 * writes one 64-byte record per ray (N*spp, ommatidium-major, sample-minor):
 * float normalDraw, uniformDraw, origin xyz, direction xyz, t, b1, b2;
 * int32 hit id (-1 = miss); float r, g, b (unscaled shaded colour); pad.
 * Advances the random streams by one frame like renderFrame.  0 on success. */
int crRenderFrameRecorded(void* records);

/* Flattened world-space scene: number of triangles, then per triangle 9
 * floats of vertices, 12 floats of colour record and one shading byte:
 * 0 = material base colour (record = the colour three times), 1 = vertex
 * colours (record = the three vertex colours), 2 = base colour texture
 * (record = (u, v, texture index, 0) per vertex).  0 on success.
 * No counterpart in the reference (test and tooling access). */
size_t crGetTriangleCount(void);
int crGetSceneTriangles(float* verts, float* colours, unsigned char* shading);

/* Decoded base colour textures of the loaded scene: texture count, total
 * texel count, then per texture (first texel, width, height) as 3 ints and
 * all texels as RGBA8 words (red in the low byte), row 0 first.  0 on
 * success.  No counterpart in the reference. */
size_t crGetTextureCount(void);
size_t crGetTexelCount(void);
int crGetSceneTextures(int* table, unsigned int* texels);

/* Samples a width x height RGBA8 texture at n (u, v) pairs with the
 * renderer's bilinear filter (rgbaRenderer) and with a CUDA texture object
 * in the reference's sampler state (rgbaHardware; wrap, linear filter,
 * normalised coordinates and reads; libEyeRenderer3/MulticamScene.cpp:800-833),
 * n x 4 floats each.  Host buffers; allocates and synchronises.  0 on
 * success.  No counterpart in the reference (sampling check). */
int crCompareTextureSampling(const unsigned int* texels, int width, int height, const float* uv, int n,
                             float* rgbaRenderer, float* rgbaHardware);

/* Current eye's ommatidium records as N x 8 floats (position, direction,
 * acceptance angle, focal offset).  0 on success. */
int crGetOmmatidia(float* out);

/* Current camera's local frame (x, y, z axes; 9 floats).  0 on success. */
int crGetCameraLocalSpace(float* axes9);

/* Current eye's generator states (8 x N*spp words, layout of the device
 * buffer).  0 on success; -1 when the streams are not initialised yet. */
int crGetRandomStates(uint32_t* out);

/* BVH statistics of the loaded scene: inner nodes, leaves, max depth. */
int crGetBvhStats(uint32_t* innerNodes, uint32_t* leaves, uint32_t* maxDepth);
}

void* getWindowPointer(); /* libEyeRenderer.h:69; there is no window: returns null */

#endif
