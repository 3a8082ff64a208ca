// Interface between the host runtime (eye_renderer.cpp) and the sm_103a
// kernels (render.cu).  Plain pointers and sizes only.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace cr {

// Device view of a scene: BVH nodes / triangles / shading records in the
// layout described in bvh.hpp.
struct DevScene {
  const float4* nodes = nullptr;
  const float4* tris = nullptr;
  const float4* shade = nullptr;
  // width 2: closest hits are searched in the two-wide BVH (nodes); 4 or 8:
  // in the wide BVH of that width with quantised child boxes (wnodes,
  // wbvh.hpp layout), over the same triangles.  The closest hit, and so every
  // result, is the same in both.
  const float4* wnodes = nullptr;
  int width = 2;
  uint32_t triCount = 0;
  int miss = 0;         // 0 = default_background, 1 = simple_sky
  float extent = 0.f;   // largest |coordinate| of any triangle vertex
  // Base-colour textures: RGBA8 texels (r in the low byte) of all textures,
  // and per texture (first texel, width, height, 0).
  const uint32_t* texels = nullptr;
  const int4* texTable = nullptr;
  // Lighting-on shading (off by default, as the reference's params.lighting):
  // per triangle in original order 5 float4 (scene.hpp's lighting layout),
  // and four point lights (position xyz + intensity; colour).
  const float4* light = nullptr;
  int lighting = 0;
  float4 lightPos[4] = {};
  float4 lightCol[4] = {};
};

// Samples one width x height RGBA8 texture at n (u, v) coordinates twice:
// with the render kernel's own bilinear filter (rgbaSoft) and with a
// hardware texture object in the reference's sampler state (wrap
// addressing, linear filtering, normalised coordinates, texels read as
// value / 255; MulticamScene.cpp:800-833) (rgbaHard).  Host buffers, n x 4
// floats out; allocates and synchronises (a check, not a render path).
cudaError_t sampleTextureBoth(const uint32_t* texels, int width, int height, const float* uv, int n, float* rgbaSoft,
                              float* rgbaHard);

// Device view of one compound eye.
//  omm: N ommatidium records of 32 bytes (2 x float4).
//  rng: XORWOW generator states, structure of arrays: 8 planes of N*spp
//       32-bit words (d, v0..v4, boxmuller_flag, boxmuller_extra); the state
//       of (ommatidium o, sample s) sits at index o*spp + s and holds the
//       stream curand_init(42, s*N + o, 0) (shaders.cu:669-695).
//  order: null, or a permutation of the N ommatidia giving the order in
//       which warp segments take them (neighbouring directions together, so
//       the rays of a warp stay coherent when it holds several ommatidia);
//       results are indexed by ommatidium and do not depend on it.
struct DevEye {
  const float4* omm = nullptr;
  uint32_t N = 0;
  uint32_t spp = 1;
  uint32_t* rng = nullptr;
  const uint32_t* order = nullptr;
  // draws: null (each warp draws its samples' random numbers pose after pose
  //       from the states it holds), or P x N x spp (normal, uniform) pairs
  //       of a launch, generated up front so that the poses of the launch can
  //       be spread over several warps (renderDrawBytes).
  float2* draws = nullptr;
  // cuts: null, or P x kCutStride float4 receiving each pose's near-field
  //       cut (render.cu, cutKernel) for a ball of radius cutRadius around
  //       the pose position; maxRel bounds |ommatidium position - focal
  //       offset along the axis| over the eye.  Results do not depend on it.
  float4* cuts = nullptr;
  float cutRadius = 0.f;
  float maxRel = 0.f;
  // netDraws: sample s of ommatidium o at pose p of the launch takes point s
  //       of a digitally shifted two-dimensional Sobol' net, the shift drawn
  //       from (drawSeed, (frame0 + p) * N + o) (render.cu, netDraw): no
  //       generator states and no pre-drawn numbers, so a launch may spread
  //       its poses over any number of warps, and each ommatidium's samples
  //       are stratified over its cone (feature renders).
  bool netDraws = false;
  unsigned long long drawSeed = 0;
  unsigned long long frame0 = 0;
};
// Traversal stack entries of the wide BVH (a node pushes up to W - 1).
constexpr int kWideStackEntries = 128;
constexpr int kCutEntries = 8;
constexpr int kCutStride = 1 + 2 * kCutEntries;

// One pose = 4 x float4: position, local x axis, local y axis, local z axis
// (w components unused).
constexpr int kPoseFloats = 16;

// Per-ray record written by the recording render variant (test and parity
// use only): draws, ray, closest hit and the unscaled shaded colour.
struct RayRecord {
  float normalDraw, uniformDraw;
  float ox, oy, oz;
  float dx, dy, dz;
  float t, b1, b2;
  int32_t hitId;  // original global triangle id, -1 on a miss
  float r, g, b;
  float pad;
};
static_assert(sizeof(RayRecord) == 64, "ray record is 64 bytes");

// Error bits raised by the kernels into a device word.
enum : uint32_t {
  kErrStackOverflow = 1u,
  kErrRngDoubleFlag = 2u,
  kErrMmaTimeout = 4u,  // a tensor-core wait ran out of its iteration limit
};

constexpr uint32_t kRngPlanes = 8;

// Samples traced by one warp segment and number of segments per ommatidium.
struct WarpPlan {
  uint32_t segWidth;     // lanes per ommatidium segment (power of two <= 32)
  uint32_t ommPerWarp;   // 32 / segWidth
  uint32_t chunks;       // warp segments per ommatidium (spp > segWidth)
  uint64_t tasks;        // warp tasks per pose batch
  uint32_t poseSplits = 1;     // pose ranges the batch is cut into (pre-drawn launches)
  uint32_t posesPerSplit = 0;  // poses per range (0: all)
  uint32_t blockWarps = 4;     // warps per block of the launch
  // inBlock: every block holds all `chunks` warps of groupsPerBlock ommatidium
  // groups and sums the chunk partials in shared memory (no scratch, no
  // second launch); tasks are then padded to whole blocks.
  uint32_t inBlock = 0;
  uint32_t groupsPerBlock = 1;
};
// The default plan: 32-sample segments (whole ommatidia when spp < 32).
WarpPlan planWarps(uint32_t N, uint32_t spp);
// Layout of the plain render kernel, process-wide (the autotuner sets it):
// block size in threads (0 = the smallest of 128, 256, 512 that holds all
// chunk warps of an ommatidium, else 128) and samples per warp segment
// (0 = 32, or 8 / 16: segments of 8 or 16 samples, several ommatidia per
// warp; a smaller segment changes the order in which samples are summed,
// so results change within float rounding).  Results never depend on the
// block size.
void setRenderLayout(uint32_t blockThreads, uint32_t samplesPerWarp);
void renderLayout(uint32_t* blockThreads, uint32_t* samplesPerWarp);
// Plan of one eye in a batched launch under that layout: its segment width,
// chunk partials in scratch (P x N x chunks x 3 floats when chunks > 1).
WarpPlan planBatch(uint32_t N, uint32_t spp);
// Block size of the batched launch (the layout's, 128 by default).
uint32_t batchBlockThreads();

// Bytes of DevEye::draws worth providing for a P-pose launch of an
// N-ommatidium, spp-sample eye: non-zero only when the eye alone has too few
// samples to fill the GPU, so that its poses are better spread over warps.
size_t renderDrawBytes(uint32_t N, uint32_t spp, uint32_t P);

// Floats of scratch needed by launchRender for P poses of the scene (0 when
// spp <= 32 or when the chunk partials are summed inside the blocks), for a
// recording (rec) or counting (stats) launch or neither; forceScratch: the
// scratch plan (chunk partials in global memory, summed by a second kernel).
size_t renderScratchFloats(const DevScene& scene, uint32_t N, uint32_t spp, uint32_t P, bool rec = false,
                           bool stats = false, bool forceScratch = false);

cudaError_t launchRngInit(const DevEye& eye, uint32_t* errFlag, cudaStream_t stream);

// Renders P poses of one eye.  out: P*N*3 floats, the per-ommatidium sums of
// sample colour / spp.  scratch: renderScratchFloats() floats or null when
// not needed.  rec: P*N*spp records or null.  stats: null, or two counters
// that receive the node visits and triangle tests of every ray.  The
// generator states advance by one frame per pose and are written back.
cudaError_t launchRender(const DevScene& scene, const DevEye& eye, const float4* poses, uint32_t P, float* out,
                         float* scratch, uint32_t* errFlag, RayRecord* rec, cudaStream_t stream,
                         unsigned long long* stats = nullptr, bool forceScratch = false);

// Per-ommatidium sample statistics of a feature render (spp <= 32), each the
// mean over the samples: colour (3), squared colour (3), hit flag, hit
// distance (0 on a miss), hit-triangle normal facing the ray in the eye's
// frame (3, 0 on a miss), and the traversal cost (BVH node visits plus
// triangle tests; the allocator's cost term).  stats: P x N x kFeatureStats
// floats.
// cutsReady: eye.cuts already holds these poses' near-field cuts (else they
// are built first when eye.cuts is set).
constexpr int kFeatureStats = 12;
constexpr int kCostStat = 11;  // index of the traversal cost in a stats row
cudaError_t launchFeatures(const DevScene& scene, const DevEye& eye, const float4* poses, uint32_t P, float* stats,
                           uint32_t* errFlag, cudaStream_t stream, bool cutsReady = false);

// Denoiser network (mlp.cu).  Feature rows are kFeatureWidth bf16 values:
// kFeatBlock values of the ommatidium itself then of its kNeighbours nearest
// neighbours, zero padded.
constexpr int kNeighbours = 6;
constexpr int kFeatBlock = 15;
constexpr int kFeatureWidth = 112;
constexpr int kMlpHidden = 128;
constexpr int kMlpOut = 8;  // 3 used

// bf16 weight matrices W[in x out] (row-major) and fp32 biases of the
// denoiser network.
struct MlpWeights {
  const __nv_bfloat16* w1;
  const __nv_bfloat16* w2;
  const __nv_bfloat16* w3;
  const __nv_bfloat16* w4;
  const float* b1;
  const float* b2;
  const float* b3;
  const float* b4;
};
static_assert(kFeatBlock * (kNeighbours + 1) <= kFeatureWidth, "feature row too narrow");

// bf16 GEMM C[M x N] = A[M x K] * B[K x N] (see mlp.cu for layouts/modes).
cudaError_t gemmBf16(int mode, int M, int N, int K, const void* A, int lda, bool aTrans, const void* B, int ldb,
                     bool bTrans, float* Cf, void* Hb, int ldc, const float* bias, const void* mask,
                     cudaStream_t stream);
// The same GEMMs on the tcgen05 tensor cores (mlp_tc.cu): 128 x 128 output
// tiles, K in chunks of 64, accumulators in TMEM.  A timed-out wait is
// recorded in a device word that takeTcGemmError reads and clears
// (kErrMmaTimeout).
cudaError_t gemmBf16Tc(int mode, int M, int N, int K, const void* A, int lda, bool aTrans, const void* B, int ldb,
                       bool bTrans, float* Cf, void* Hb, int ldc, const float* bias, const void* mask,
                       cudaStream_t stream);
cudaError_t takeTcGemmError(uint32_t* flags);
cudaError_t colSumBf16(const void* in, int M, int N, int ld, float* out, cudaStream_t stream);
cudaError_t colSumF32(const float* in, int M, int N, int ld, float* out, cudaStream_t stream);
// Position of a training loop on the device.  The kernels of one step read
// it, so that one captured step can be replayed as a CUDA graph.
struct TrainState {
  int step;         // index into the step-size schedule and the loss array
  uint32_t offset;  // first entry of this step's rows in the shuffled order
};
// lossIndex: null, or the device index added to lossSum.
cudaError_t mlpLoss(const float* y, int ldy, const float* base, const float* target, int rows, float* pred, float* dyf,
                    void* dyb, float* lossSum, cudaStream_t stream, const int* lossIndex = nullptr);
// state->step += 1, state->offset += rows.
cudaError_t advanceTrainState(TrainState* state, uint32_t rows, cudaStream_t stream);
// Row-major weight matrices inside a flat parameter vector.  Their
// transposes (same offsets) are the K-contiguous operands of the tcgen05
// forward GEMMs.
struct WeightBlocks {
  int count;
  int off[4], rows[4], cols[4];
};
// Adam on the fp32 master weights; refreshes the bf16 copy wb and, when
// wbT is given, the bf16 transposes of `blocks` in wbT.  sched: null, or
// per step (step size, 1 / (1 - b1^t), 1 / (1 - b2^t)) on the device, read
// at the device index *stepIdx in place of lr and t.
cudaError_t adamStep(float* w, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                     int t, void* wb, cudaStream_t stream, void* wbT = nullptr, const WeightBlocks* blocks = nullptr,
                     const float* sched = nullptr, const int* stepIdx = nullptr);
// wbT = bf16 transposes of `blocks` of the n fp32 parameters w.
cudaError_t transposeWeightsBf16(const float* w, size_t n, void* wbT, const WeightBlocks& blocks, cudaStream_t stream);
cudaError_t toBf16(const float* in, void* out, size_t n, cudaStream_t stream);
cudaError_t nearestOmmatidia(const float4* omm, uint32_t N, int* nb, cudaStream_t stream);
cudaError_t assembleFeatures(const float* stats, const float4* omm, const int* nb, uint32_t N, uint32_t P, void* X,
                             float* base, cudaStream_t stream);
// Fused prediction for P poses of an N-ommatidium eye straight from the
// feature-render statistics: out (P x N x 3) = own mean colour + network
// output (or the network output alone when !residual), bit-identical to
// assembleFeatures + the layer-by-layer forward.
cudaError_t inferDenoiser(const float* stats, const float4* omm, const int* nb, uint32_t N, uint32_t P,
                          const MlpWeights& w, float* out, cudaStream_t stream, bool residual = true);
// The bounded-wait path of the tcgen05 kernels, on its own (mlp_tc.cu): one
// block waits on an mbarrier that nothing arrives on, for `polls` polls, then
// sets kErrMmaTimeout in errFlag and returns.
cudaError_t launchWaitProbe(uint32_t polls, uint32_t* errFlag, cudaStream_t stream);
// Inputs of the tcgen05 prediction (mlp_tc.cu): per row of the P x N
// statistics three float4 of derived values (derived: 3 N P float4), per
// ommatidium its unit axis and acceptance angle (axes: N float4).
cudaError_t deriveFeatureStats(const float* stats, const float4* omm, uint32_t N, uint32_t P, float4* derived,
                               float4* axes, cudaStream_t stream);
// The same prediction on the tcgen05 tensor cores (mlp_tc.cu) from
// deriveFeatureStats' output: accumulators in TMEM, operands in shared
// memory; errFlag receives kErrMmaTimeout if a bounded wait ran out.  order:
// null, or the eye's direction order (rows of a tile are then neighbouring
// ommatidia; results do not depend on it).
cudaError_t inferDenoiserTc(const float4* derived, const float4* axes, const int* nb, uint32_t N, uint32_t P,
                            const MlpWeights& w, float* out, uint32_t* errFlag, cudaStream_t stream,
                            bool residual = true, const uint32_t* order = nullptr);
// Rows idx[offset .. offset + rows) of the training set, offset = *offset
// on the device when given, else 0.
cudaError_t gatherRows(const void* X, const float* base, const float* target, const uint32_t* idx, int rows, void* Xo,
                       float* baseo, float* targeto, cudaStream_t stream, const uint32_t* offset = nullptr);

// Tuning variants of the plain render kernel (see render.cu); the variant
// is process-wide and picked by the autotuner in eye_renderer.cpp.
int renderVariantCount();
void setRenderVariant(int v);
int renderVariant();

// GPU BVH construction (lbvh.cu): bytes of temporary device memory for T
// triangles, and the build itself.  verts: 9 floats, colours: 12 floats,
// flags: 1 byte per triangle (device).  centroidLo/Hi: host bounds of the
// triangle-box centres.  nodes: (T-1) x 4 float4, tris/shade: T x 3 float4.
// statsOut (host): inner nodes, leaf references, maximum leaf depth.
// Requires T >= 9; synchronises the stream.
size_t lbvhTempBytes(uint32_t T);
cudaError_t buildLbvh(const float* d_verts, const float* d_colours, const uint8_t* d_flags, uint32_t T,
                      const float* centroidLo, const float* centroidHi, float4* d_nodes, float4* d_tris,
                      float4* d_shade, void* d_temp, uint32_t* statsOut, cudaStream_t stream);

// One eye of a batched launch (device table entry).
struct BatchEye {
  DevEye eye;
  const float4* poses;  // P poses of this eye
  float* out;           // P x N x 3
  float* scratch;       // P x N x chunks x 3, or null when chunks == 1
  WarpPlan plan;
  uint32_t P;
};

// Resident blocks per SM of the batch kernel for a render variant.
int batchBlocksPerSM(int variant);

// Persistent launch over all eyes' warp tasks (taskBase: nEyes ascending
// task offsets) followed by the chunk sums of the eyes with chunks > 1
// (cellBase: nEyes ascending offsets into their P*N cells).  ctrl must hold
// 2 + nEyes words, set to {0, ~0, 0...} before the launch.  cutPoses > 0:
// first build the near-field cuts of the eyes whose DevEye::cuts is set
// (cutPoses poses per eye, each eye's cuts laid out like a plain launch's).
cudaError_t launchBatch(const DevScene& scene, const BatchEye* eyes, const unsigned long long* taskBase,
                        const unsigned long long* cellBase, uint32_t nEyes, unsigned long long totalTasks,
                        unsigned long long totalCells, unsigned long long* ctrl, uint32_t* errFlag, int variant,
                        int gridBlocks, uint32_t cutPoses, cudaStream_t stream);

// Adaptive sampling (render.cu).  An entry e = pose * N + ommatidium is
// rendered at its bucket's sample count; buckets hold counts 4 << index.
constexpr uint32_t kAdaptiveBuckets = 9;  // 4, 8, ..., 1024
constexpr uint8_t kNoRender = 0xFF;        // level of an entry the feature render covers
#ifdef __CUDACC__
#define CR_HOST_DEVICE __host__ __device__
#else
#define CR_HOST_DEVICE
#endif
// Samples each lane traces per task (up to 8, for counts above 32) and warp
// tasks per entry of a bucket with `spp` samples (a power of two).
CR_HOST_DEVICE inline uint32_t adaptiveSamplesPerLane(uint32_t spp) {
  return spp <= 32 ? 1u : (spp / 32 < 8 ? spp / 32 : 8u);
}
CR_HOST_DEVICE inline uint32_t adaptiveChunks(uint32_t spp) {
  return spp <= 32 ? 1u : spp / (32u * adaptiveSamplesPerLane(spp));
}
struct AdaptiveBucket {
  const uint32_t* entries = nullptr;  // count entry ids
  uint64_t count = 0;
  uint32_t spp = 0;
  float* partials = nullptr;  // adaptivePartialFloats(count, spp) floats when spp > 32
  uint64_t taskBase = 0;      // first warp task of the bucket
  uint64_t tasks = 0;         // warp tasks of the bucket
  uint64_t poolBase = 0;      // first warp pool of the bucket (a pool: up to 8 rounds of 32 samples)
};
struct AdaptiveLaunch {
  AdaptiveBucket b[kAdaptiveBuckets];
  uint32_t nBuckets = 0;
  uint64_t totalTasks = 0;
  uint64_t totalPools = 0;
  // Ray refill: a warp hands its idle lanes new samples once at least
  // refillIdle of its 32 lanes are idle, checking every `steps` BVH steps.
  uint32_t refillIdle = 16;
  int steps = 16;
  // Resident 128-thread blocks per SM the kernel's register budget is sized
  // for on the two-wide BVH: 5 (96 registers), 6 (80) or 8 (64).
  int blocksPerSM = 5;
};
// Table of the non-empty buckets among nBuckets (entries, counts, spp and
// partial buffers per bucket) with their warp-task offsets.
AdaptiveLaunch planAdaptive(const uint32_t* const* entries, const uint64_t* counts, const uint32_t* spp,
                            float* const* partials, uint32_t nBuckets);
// The process-wide ray-refill schedule of the adaptive kernel (planAdaptive
// copies it into every launch): refill at >= refillIdle idle lanes (1..32),
// check every `steps` BVH steps (1..4096).  Results do not depend on it.
void setAdaptiveSchedule(uint32_t refillIdle, int steps);
void adaptiveSchedule(uint32_t* refillIdle, int* steps);
// The process-wide occupancy of the adaptive kernel (5, 6 or 8 blocks per
// SM; other values mean 5).  Results do not depend on it.
void setAdaptiveBlocksPerSM(int blocks);
int adaptiveBlocksPerSM();
size_t adaptivePartialFloats(uint64_t count, uint32_t spp);
// One launch over every bucket: sums[3e..3e+2] = mean sample colour of entry
// e, its samples the points of a digitally shifted Sobol' net keyed by
// (seed, e) (render.cu, netDraw).  rec:
// null, or count x spp records of a single-bucket launch (tests).
cudaError_t launchAdaptive(const DevScene& scene, const float4* omm, uint32_t N, const float4* poses,
                           const AdaptiveLaunch& L, unsigned long long seed, float* sums, uint32_t* errFlag,
                           RayRecord* rec, cudaStream_t stream, const float4* cuts = nullptr);
// isInsideHitGeometry for n points (xyz floats) against one hitbox mesh
// (object-space triangles, 3 float3 each): the inverse of the 3x3 part of
// the mesh's node transform (row-major, double; the object-space point is
// rounded once to float; as in the reference, the node's translation does
// not enter) and the ray start x = object box min.x - 1
// (a float value); the cast itself runs in float as the reference's
// (sutil/hitscanprocessing.cpp:20-83).  out: one byte per point, 1 = inside.
struct InsideQuery {
  double inv[9];
  double startX;
  // Grid over the object-space (y, z) plane: cell (cz * G + cy) lists, in
  // cellItems[cellStart[c] .. cellStart[c + 1]), every triangle whose (y, z)
  // box, widened by a margin, meets the cell; cell of y is
  // floor((y - y0) * inv) clamped to [0, G).  G == 0: test every triangle.
  const uint32_t* cellStart = nullptr;
  const uint32_t* cellItems = nullptr;
  // Triangles whose cast normal is not finite (zero area): their test does
  // not depend on the point, so with a grid they are tested for every point
  // (they are in no cell).
  const uint32_t* everywhere = nullptr;
  uint32_t nEverywhere = 0;
  double y0 = 0.0, z0 = 0.0, cellInv = 0.0;
  int G = 0;
};
cudaError_t launchInside(const float3* tris, uint32_t nTris, const InsideQuery& q, const float* pts, size_t n,
                         uint8_t* out, cudaStream_t stream);
// Near-field cuts of P poses (kCutStride float4 each; see DevEye::cuts).
cudaError_t launchCuts(const DevScene& scene, const float4* poses, uint32_t P, float radius, float maxRel,
                       float4* cuts, cudaStream_t stream);
// Minimum-sample labels: entries with label 0 get `spp` when the standard
// deviation across the k renders outs[k][rows][3] is below thr in every channel.
cudaError_t launchLabels(const float* outs, int k, uint64_t rows, uint32_t spp, float thr, uint16_t* label,
                         cudaStream_t stream);
// Per-entry bucket level from the allocator's prediction (rows x 3) and the
// bucket sizes (counts: kAdaptiveBuckets words, zeroed by the caller);
// the count rendered is 2^(exponent * log2(predicted count) - halvings -
// costExponent * log2(cost / kCostRef)), cost the entry's traversal cost
// from the feature statistics (stats: rows x kFeatureStats; unused when
// costExponent is 0).
constexpr float kCostRef = 16.0f;
cudaError_t launchAllocate(const float* pred, uint64_t rows, uint32_t featureSpp, uint8_t* level,
                           unsigned long long* counts, cudaStream_t stream, float halvings = 0.f,
                           float exponent = 1.f, const float* stats = nullptr, float costExponent = 0.f);
// Entry lists of rows = P x N entries, pose by pose and within a pose in the
// eye's `order` (null: index order): bucket k's entries go to
// entries[bucketBase[k]...] (bucketBase: device, kAdaptiveBuckets words);
// scratch: scatterScratchWords(rows) words.
size_t scatterScratchWords(uint64_t rows);
cudaError_t launchScatterBuckets(const uint8_t* level, uint64_t rows, uint32_t N, const uint32_t* order,
                                 const unsigned long long* bucketBase, unsigned long long* scratch, uint32_t* entries,
                                 cudaStream_t stream);
// Final colours of an adaptive render (see render.cu).
cudaError_t launchAdaptiveFinish(const uint8_t* level, uint64_t rows, uint32_t featureSpp, const float* stats,
                                 const float* learned, const float* sums, float* out, cudaStream_t stream);

// Fixed device array used as render scratch by the allocation-free entry
// point: its capacity in floats, and its address on the current device
// (looked up on the first call per device).
size_t noAllocScratchFloats();
cudaError_t noAllocScratch(float** ptr);

// Projection of per-ommatidium sums into a w x h uchar4 frame.
//  mode 0: single_dimension_fast (row 0, x < N), mode 1: single_dimension.
cudaError_t launchProject(const float* sums, uint32_t N, uchar4* frame, int w, int h, int mode,
                          cudaStream_t stream);
// Candidates of the spherical projections binned by unit vector: a G^3 grid
// over [-1, 1]^3, cell (cz * G + cy) * G + cx holding items[start[c] ..
// start[c + 1]) (ommatidium indices >= 1, ascending).  G == 0: no candidate.
struct SphereGridView {
  const uint32_t* start = nullptr;  // G^3 + 1 offsets
  const uint32_t* items = nullptr;
  int G = 0;
};
// The four candidate sets: 0 positions, 1 directions, 2 directions of the
// ommatidia with position.x < 0, 3 those with position.x > 0.
struct SphereGridSet {
  SphereGridView g[4];
};

// Spherical projections (kind: 0 positionwise, 1 orientationwise, 2 split
// orientationwise, 3 orientationwise ids, 4 positionwise ids); lenScratch
// holds 2 * N floats.  grids: the candidate grids (searched around each
// pixel's point), or null for the exhaustive search in index order; both
// give the same image.
cudaError_t launchSpherical(const float4* omm, float* lenScratch, uint32_t N, const float* sums, uchar4* frame, int w,
                            int h, int kind, const SphereGridSet* grids, cudaStream_t stream);
// raw_ommatidial_samples from a recorded frame (N x spp records).
cudaError_t launchRawSamples(const RayRecord* rec, uint32_t N, uint32_t spp, uchar4* frame, int w, int h,
                             cudaStream_t stream);

}  // namespace cr
