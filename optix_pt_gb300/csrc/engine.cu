// The renderer behind the C ABI (include/optpt.h): scene upload, GPU BVH
// build, wavefront buffers, the CUDA-graph-captured bounce loop, and the
// parity entry points. Replaces the reference's Renderer
// (src/renderer.cpp:24-1762) minus OptiX set-up, denoiser and GL display.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>
#include "../../include/optpt.h"
#include "engine.h"
#include "image_io.h"
#include "guide_net.h"

int uploadSrgbTable();

namespace {

thread_local std::string g_lastError;

int fail(int code, const std::string &msg)
{
    g_lastError = msg;
    return code;
}

int cudaFail(cudaError_t e, const char *where)
{
    return fail(OPTPT_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CUDA_OR_RETURN(expr, where)                                                                                    \
    do {                                                                                                               \
        cudaError_t e_ = (expr);                                                                                       \
        if (e_ != cudaSuccess)                                                                                         \
            return cudaFail(e_, where);                                                                                \
    } while (0)

template <class T> cudaError_t upload(T *&dst, const T *src, size_t count)
{
    dst = nullptr;
    if (count == 0 || src == nullptr)
        return cudaSuccess;
    cudaError_t e = cudaMalloc((void **)&dst, sizeof(T) * count);
    if (e != cudaSuccess)
        return e;
    return cudaMemcpy(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
}

}  // namespace

struct optpt_renderer {
    // scene (device)
    float *dPositions = nullptr, *dNormals = nullptr, *dTexCoords = nullptr;
    int *dTriIndices = nullptr, *dMatIndices = nullptr;
    uint32_t *dTriFlags = nullptr;
    DevMaterial *dMaterials = nullptr;
    DevLight *dLights = nullptr;
    Light *dLightsPublic = nullptr;
    float4 *dEmisV = nullptr, *dEmisRad = nullptr;
    float2 *dEmisTc = nullptr;
    uint32_t *dTexels = nullptr;
    int4 *dTexInfo = nullptr;
    BvhBuild bvh{};
    DevScene scene{};
    int numTris = 0, numEmissive = 0, numLights = 0;

    // frame
    LaunchParams lp{};
    optpt_options opt{};
    uint32_t w = 0, h = 0, sppBatch = 1;
    WaveBufs q{};
    AccumBufs acc{};
    uint32_t *dState = nullptr;
    LaunchShape shape{};
    std::vector<float> hostFb;
    bool hostFbValid = false;
    // Pipelined launches (optpt_launch_pipelined): a frame's tone-mapped
    // buffer is snapshot on the device and copied to pinned host memory on a
    // copy stream while the next frame renders; two slots alternate.
    struct FramePipe {
        float4 *stage[2] = {nullptr, nullptr};
        float *host[2] = {nullptr, nullptr};
        cudaEvent_t staged[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
        cudaStream_t copyStream = nullptr;
        size_t pixels = 0;
        uint32_t next = 0;  // slot of the next frame
        int pending = -1;   // slot whose copy is in flight, -1 = none
    } pipe;
    void *outScratch = nullptr;  // device payloads of optpt_read_rgba8 / optpt_save_image
    size_t outScratchBytes = 0;

    // deformation (optpt_set_deformation / optpt_deform / optpt_update_vertices)
    uint32_t numVerts = 0;
    int *dEmisPrim = nullptr;
    float *dRestPos = nullptr, *dRestNrm = nullptr, *dShapeM = nullptr, *dShapeN = nullptr, *dJointM = nullptr;
    uint32_t *dVShape = nullptr;
    void *dJoints = nullptr, *dWeights = nullptr;
    uint32_t defVerts = 0, defShapes = 0, defJoints = 0;
    bool hasNormals = false;

    // graph of one pass, re-captured when the frame parameters change
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graphExec = nullptr;
    bool graphDirty = true;
    cudaStream_t ownStream = nullptr;
    // Side stream of a pass: each bounce's shadow launches run on it, beside
    // the next bounce's extension (fork after shading, join before the next
    // shading).
    cudaStream_t sideStream = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;

    FrameConst *dFrameConst = nullptr;
    // Frame constants go up from a small pinned ring: an upload from pageable
    // memory may wait for the stream's earlier work (the driver stages it),
    // which would leave the GPU idle while the host enqueues the next frame.
    // A slot is rewritten only after its previous copy has run.
    static constexpr int FC_SLOTS = 4;
    FrameConst *hFrameConst = nullptr;  // pinned, FC_SLOTS entries
    cudaEvent_t fcCopied[FC_SLOTS] = {};
    uint32_t fcNext = 0;

    // learned guiding (mode 0 off, 1 guided + online training, 2 guided, frozen)
    optpt_guide *guide = nullptr;
    int guideMode = 0;
    // First bounce finished by the path-completion kernel (plain sampling);
    // 0 = every bounce by the per-bounce kernels.
    uint32_t tailBounce = 0;
    void *gMix = nullptr;        // 80 B per path slot
    float4 *gRec = nullptr;      // GUIDE_REC float4 per (training path, depth)
    void *gBatch = nullptr;      // GuideSample per slot
    uint32_t *gBatchCount = nullptr;
    size_t gMixPaths = 0, gRecSlots = 0;
    uint32_t gTrainStride = 1, gBatchCap = 1u << 18, gTrainSteps = 4, gMaxDepth = 0xFFFFFFFFu;
    uint32_t gTrainSpp = 0xFFFFFFFFu;  // online training stops after this many samples per pixel
    bool gSharePrimary = false;        // a pixel's primary hits share one mixture per pass
    uint64_t gTrainedSpp = 0;          // samples per pixel rendered with training so far
    bool graphTrain = false;           // training state the captured pass was recorded with
    bool trainingOpen() const { return guideMode == 1 && gTrainedSpp < gTrainSpp; }
    float gAlphaMin = 0.0f, gAlphaMax = 0.6f, gAlphaRamp = 64.0f, gLr = 1e-2f;
    int gLobeLoss = 1;
    float sceneLo[3] = {0, 0, 0}, sceneHi[3] = {0, 0, 0};

    // batched multi-view rendering (optpt_render_batch)
    struct Batch {
        WaveBufs q{};
        AccumBufs acc{};
        BatchView *dViews = nullptr;
        uint32_t *dPixelList = nullptr, *dDyn = nullptr;
        uint16_t *dPixelView = nullptr;
        std::vector<optpt_view> views;
        std::vector<uint32_t> first, done;
        uint32_t totalPixels = 0, maxPaths = 0, maxDepth = 0;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        int guideMode = -1;
        // per-pass host state (batchPassSizes)
        std::vector<char> wasActive;
        std::vector<uint32_t> list;
        std::vector<BatchView> hostViews;
        uint32_t per = 0;
        uint32_t dyn[2] = {0, 0};
    } batch;

    void freeBatch()
    {
        Batch &b = batch;
        if (b.exec)
            cudaGraphExecDestroy(b.exec);
        if (b.graph)
            cudaGraphDestroy(b.graph);
        float4 *bufs[] = {b.q.pathT, b.q.pathL, b.q.rayO[0], b.q.rayO[1], b.q.rayD[0], b.q.rayD[1], b.q.hit,
                          b.q.shO[0], b.q.shO[1], b.q.shD[0], b.q.shD[1], b.q.shC[0], b.q.shC[1],
                          b.acc.frameBuffer, b.acc.accumFrameBuffer};
        for (float4 *p : bufs)
            cudaFree(p);
        cudaFree(b.acc.sum);
        cudaFree(b.acc.sumSq);
        cudaFree(b.dViews);
        cudaFree(b.dPixelList);
        cudaFree(b.dDyn);
        cudaFree(b.dPixelView);
        batch = Batch{};
    }

    FrameParams frameParams() const
    {
        FrameParams fp{};
        fp.w = w;
        fp.h = h;
        fp.npix = w * h;
        fp.sppBatch = sppBatch;
        fp.numPaths = w * h * sppBatch;
        fp.maxDepth = lp.maxDepth;
        fp.state = dState;
        fp.fc = dFrameConst;
        if (guideMode != 0) {
            fp.guide.mix = gMix;
            fp.guide.rec = gRec;
            fp.guide.batch = gBatch;
            fp.guide.batchCount = gBatchCount;
            fp.guide.on = 1;
            fp.guide.train = trainingOpen() ? 1u : 0u;
            fp.guide.trainStride = gTrainStride;
            fp.guide.batchCapacity = gBatchCap;
            fp.guide.step = guide->dStep;
            fp.guide.alphaMin = gAlphaMin;
            fp.guide.alphaMax = gAlphaMax;
            fp.guide.alphaRamp = gAlphaRamp;
            fp.guide.maxDepth = gMaxDepth;
            fp.guide.sharePrimary = gSharePrimary ? 1u : 0u;
        }
        return fp;
    }

    void freeGuideBuffers()
    {
        cudaFree(gMix);
        cudaFree(gRec);
        cudaFree(gBatch);
        cudaFree(gBatchCount);
        gMix = nullptr;
        gRec = nullptr;
        gBatch = nullptr;
        gBatchCount = nullptr;
        gMixPaths = gRecSlots = 0;
    }

    cudaError_t uploadFrameConst(cudaStream_t st)
    {
        const uint32_t k = fcNext;
        fcNext = (k + 1) % FC_SLOTS;
        cudaError_t e = cudaEventSynchronize(fcCopied[k]);  // returns at once if never recorded
        if (e != cudaSuccess)
            return e;
        hFrameConst[k] = frameConst();
        if ((e = cudaMemcpyAsync(dFrameConst, hFrameConst + k, sizeof(FrameConst), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            return e;
        return cudaEventRecord(fcCopied[k], st);
    }

    FrameConst frameConst() const
    {
        auto bits = [](uint32_t u) {
            float f;
            memcpy(&f, &u, 4);
            return f;
        };
        FrameConst c;
        c.eye = make_float4(lp.eye[0], lp.eye[1], lp.eye[2], bits(lp.seed));
        c.U = make_float4(lp.U[0], lp.U[1], lp.U[2], bits((uint32_t)lp.vis));
        const uint32_t tone = (lp.toneMapping ? 1u : 0u) | (lp.toneMappingImpl ? 2u : 0u) | (lp.gammaCorrection ? 4u : 0u);
        c.V = make_float4(lp.V[0], lp.V[1], lp.V[2], bits(tone));
        c.W = make_float4(lp.W[0], lp.W[1], lp.W[2], lp.gammaTerm);
        c.bg = make_float4(lp.bgColour[0], lp.bgColour[1], lp.bgColour[2], 0.0f);
        return c;
    }

    void freePipe()
    {
        if (pipe.copyStream)
            cudaStreamSynchronize(pipe.copyStream);
        for (int k = 0; k < 2; ++k) {
            cudaFree(pipe.stage[k]);
            if (pipe.host[k])
                cudaFreeHost(pipe.host[k]);
            if (pipe.staged[k])
                cudaEventDestroy(pipe.staged[k]);
            if (pipe.copied[k])
                cudaEventDestroy(pipe.copied[k]);
        }
        if (pipe.copyStream)
            cudaStreamDestroy(pipe.copyStream);
        pipe = FramePipe{};
    }

    void freeFrame()
    {
        freePipe();
        if (graphExec)
            cudaGraphExecDestroy(graphExec);
        if (graph)
            cudaGraphDestroy(graph);
        graphExec = nullptr;
        graph = nullptr;
        graphDirty = true;
        cudaFree(q.pathT);
        cudaFree(q.pathL);
        for (int k = 0; k < 2; ++k) {
            cudaFree(q.rayO[k]);
            cudaFree(q.rayD[k]);
            cudaFree(q.shO[k]);
            cudaFree(q.shD[k]);
            cudaFree(q.shC[k]);
        }
        cudaFree(q.hit);
        cudaFree(acc.sum);
        cudaFree(acc.sumSq);
        cudaFree(acc.frameBuffer);
        cudaFree(acc.accumFrameBuffer);
        unsigned long long *totals = q.totals;
        uint32_t *counters = q.counters;
        q = WaveBufs{};
        q.totals = totals;
        q.counters = counters;
        acc = AccumBufs{};
    }

    ~optpt_renderer()
    {
        freeFrame();
        freeBatch();
        freeGuideBuffers();
        if (guide) {
            guideFree(guide);
            delete guide;
        }
        cudaFree(q.totals);
        cudaFree(q.counters);
        cudaFree(dState);
        cudaFree(dFrameConst);
        if (hFrameConst)
            cudaFreeHost(hFrameConst);
        for (auto &e : fcCopied)
            if (e)
                cudaEventDestroy(e);
        freeBvh(bvh);
        cudaFree(dPositions);
        cudaFree(dNormals);
        cudaFree(dTexCoords);
        cudaFree(dTriIndices);
        cudaFree(dMatIndices);
        cudaFree(dTriFlags);
        cudaFree(dMaterials);
        cudaFree(dLights);
        cudaFree(dLightsPublic);
        cudaFree(dEmisV);
        cudaFree(dEmisRad);
        cudaFree(dEmisTc);
        cudaFree(dTexels);
        cudaFree(dTexInfo);
        cudaFree(outScratch);
        cudaFree(dEmisPrim);
        cudaFree(dRestPos);
        cudaFree(dRestNrm);
        cudaFree(dShapeM);
        cudaFree(dShapeN);
        cudaFree(dJointM);
        cudaFree(dVShape);
        cudaFree(dJoints);
        cudaFree(dWeights);
        if (evFork)
            cudaEventDestroy(evFork);
        if (evJoin)
            cudaEventDestroy(evJoin);
        if (sideStream)
            cudaStreamDestroy(sideStream);
        if (ownStream)
            cudaStreamDestroy(ownStream);
    }
};

namespace {

// Camera::setParams + setupUvwCoordinatSystem (src/camera.cpp:6-40).
void cameraBasis(const float eye[3], const float target[3], const float up[3], float fovYDeg, float aspect,
                 float U[3], float V[3], float W[3])
{
    auto nrm = [](double v[3]) {
        double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        v[0] /= l;
        v[1] /= l;
        v[2] /= l;
    };
    auto crs = [](const double a[3], const double b[3], double o[3]) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    double w[3] = {(double)target[0] - eye[0], (double)target[1] - eye[1], (double)target[2] - eye[2]};
    nrm(w);
    double upn[3] = {up[0], up[1], up[2]};
    nrm(upn);
    double mw[3] = {-w[0], -w[1], -w[2]}, u[3], v[3];
    crs(upn, mw, u);
    nrm(u);
    crs(mw, u, v);
    nrm(v);
    const double vLen = std::tan(0.5 * fovYDeg * 3.14159265358979323846 / 180.0);
    const double uLen = vLen * aspect;
    for (int k = 0; k < 3; ++k) {
        U[k] = (float)(u[k] * uLen);
        V[k] = (float)(v[k] * vLen);
        W[k] = (float)w[k];
    }
}

int allocFrame(optpt_renderer *r, uint32_t width, uint32_t height)
{
    r->freeFrame();
    r->w = width;
    r->h = height;
    const size_t npix = (size_t)width * height;
    uint32_t b = r->opt.sppBatch;
    if (b == 0) {
        b = (uint32_t)((1u << 21) / (npix ? npix : 1));
        b = b < 1 ? 1 : (b > 64 ? 64 : b);
    }
    r->sppBatch = b;
    const size_t P = npix * b;
    auto al = [&](float4 *&p, size_t n) { return cudaMalloc((void **)&p, sizeof(float4) * (n ? n : 1)); };
    CUDA_OR_RETURN(al(r->q.pathT, P), "alloc pathT");
    CUDA_OR_RETURN(al(r->q.pathL, P), "alloc pathL");
    for (int k = 0; k < 2; ++k) {
        CUDA_OR_RETURN(al(r->q.rayO[k], P), "alloc rays");
        CUDA_OR_RETURN(al(r->q.rayD[k], P), "alloc rays");
        CUDA_OR_RETURN(al(r->q.shO[k], P), "alloc shadow rays");
        CUDA_OR_RETURN(al(r->q.shD[k], P), "alloc shadow rays");
        CUDA_OR_RETURN(al(r->q.shC[k], P), "alloc shadow rays");
    }
    CUDA_OR_RETURN(al(r->q.hit, P), "alloc hits");
    CUDA_OR_RETURN(cudaMalloc((void **)&r->acc.sum, sizeof(Acc4) * (npix ? npix : 1)), "alloc accum");
    CUDA_OR_RETURN(cudaMalloc((void **)&r->acc.sumSq, sizeof(Acc4) * (npix ? npix : 1)), "alloc accum");
    CUDA_OR_RETURN(al(r->acc.frameBuffer, npix), "alloc frameBuffer");
    CUDA_OR_RETURN(al(r->acc.accumFrameBuffer, npix), "alloc accumFrameBuffer");
    CUDA_OR_RETURN(cudaMemset(r->acc.sum, 0, sizeof(Acc4) * npix), "clear accum");
    CUDA_OR_RETURN(cudaMemset(r->acc.sumSq, 0, sizeof(Acc4) * npix), "clear accum");
    CUDA_OR_RETURN(cudaMemset(r->acc.frameBuffer, 0, sizeof(float4) * npix), "clear fb");
    CUDA_OR_RETURN(cudaMemset(r->acc.accumFrameBuffer, 0, sizeof(float4) * npix), "clear fb");
    CUDA_OR_RETURN(cudaMemset(r->dState, 0, sizeof(uint32_t)), "clear state");
    r->lp.sample = 0;
    r->lp.w = width;
    r->lp.h = height;
    r->lp.frameBuffer = (float *)r->acc.frameBuffer;
    r->lp.accumFrameBuffer = (float *)r->acc.accumFrameBuffer;
    r->hostFb.assign(npix * 4, 0.0f);
    r->hostFbValid = false;
    const int blk = r->opt.blockSize ? (int)r->opt.blockSize : 128;
    r->shape.block = blk;
    r->shape.compaction = r->opt.compaction == 1 ? 1 : 0;
    r->shape.gridGenerate = occupancyGrid(0, blk);
    const bool wide = r->bvh.nodes8 != nullptr;
    r->shape.gridExtend = occupancyGrid(wide ? 1 : 11, blk);
    r->shape.gridShade = occupancyGrid(2, blk);
    r->shape.gridShadow = occupancyGrid(wide ? 3 : 13, blk);
    r->shape.gridAccum = occupancyGrid(4, blk);
    r->shape.gridFinish = occupancyGrid(wide ? 5 : 15, 128);
    r->graphDirty = true;
    return OPTPT_OK;
}

// One pass: sppBatch samples for every pixel.
// Returns the number of events recorded (profiling), each tagged in `kind`.
int enqueuePassOn(optpt_renderer *r, const FrameParams &fp, const WaveBufs &q, const AccumBufs &acc, cudaStream_t st,
                  cudaEvent_t *ev, int *kind, bool count = false)
{
    int e = 0;
    auto mark = [&](int k) {
        if (ev) {
            cudaEventRecord(ev[e], st);
            kind[e] = k;
            ++e;
        }
    };
    cudaMemsetAsync(q.counters, 0, sizeof(uint32_t) * CNT_TOTAL, st);
    if (fp.guide.train)
        cudaMemsetAsync(fp.guide.batchCount, 0, sizeof(uint32_t), st);
    // Bounce d's shadow rays and bounce d + 1's extension rays are
    // independent (the shadow launches add to the path radiance, which only
    // the next shading reads), so the shadow launches go to the side stream
    // and overlap the next extension (and inference). Past the first bounces
    // the queues are short and every launch is bound by its longest ray, so
    // running them side by side hides one behind the other. Timed profiling
    // and the counting variant keep one stream.
    const bool fork = ev == nullptr && !count && r->sideStream != nullptr;
    mark(0);
    launchGenerate(r->shape, fp, q, st);
    // From bounce tailBounce on, one launch finishes every remaining path
    // (launchFinish) instead of a launch per kernel per bounce. It samples
    // the BSDF only, so with guiding on it starts past the guided bounces:
    // at guide.maxDepth + 1 at the earliest, and at guide.maxDepth + 2 while
    // the network trains, since the shading of bounce guide.maxDepth + 1 then
    // writes the arrival record of a training path's last guided vertex.
    uint32_t tail = r->tailBounce;
    if (fp.guide.on && tail != 0u)
        tail = fp.guide.maxDepth < OPT_MAX_DEPTH
                   ? std::max(tail, fp.guide.maxDepth + (fp.guide.train ? 2u : 1u))
                   : 0u;
    for (uint32_t d = 1; d <= fp.maxDepth; ++d) {
        if (d == tail) {
            if (fork && d > 1)
                cudaStreamWaitEvent(st, r->evJoin, 0);  // bounce d - 1's shadow rays resolved
            mark(7);
            launchFinish(r->shape, r->scene, fp, q, (int)d, st, count);
            break;
        }
        mark(1);
        launchExtend(r->shape, r->scene, fp, q, (int)d, st, count);
        if (fp.guide.on && d < fp.maxDepth && d <= fp.guide.maxDepth) {
            mark(5);
            launchGuideInfer(r->guide, r->scene, fp, q, (int)d, st);
        }
        if (fork && d > 1)
            cudaStreamWaitEvent(st, r->evJoin, 0);  // bounce d - 1's shadow rays resolved
        mark(2);
        launchShade(r->shape, r->scene, fp, q, (int)d, st);
        mark(3);
        if (fork) {
            cudaEventRecord(r->evFork, st);
            cudaStreamWaitEvent(r->sideStream, r->evFork, 0);
            launchShadow(r->shape, r->scene, fp, q, (int)d, 0, r->sideStream, count);
            launchShadow(r->shape, r->scene, fp, q, (int)d, 1, r->sideStream, count);
            cudaEventRecord(r->evJoin, r->sideStream);
        } else {
            launchShadow(r->shape, r->scene, fp, q, (int)d, 0, st, count);
            launchShadow(r->shape, r->scene, fp, q, (int)d, 1, st, count);
        }
    }
    if (fork)
        cudaStreamWaitEvent(st, r->evJoin, 0);  // the last bounce's shadow rays
    if (fp.guide.train) {
        // online training on this pass's samples (before the pass count advances)
        mark(6);
        launchGuideGather(fp, q, st);
        for (uint32_t k = 0; k < r->gTrainSteps; ++k) {  // minibatches of the pass's samples
            guideGradients(r->guide, reinterpret_cast<const GuideSample *>(fp.guide.batch), fp.guide.batchCount,
                           fp.guide.batchCapacity, st, k, r->gTrainSteps);
            guideAdam(r->guide, st);
        }
    }
    mark(4);
    launchAccumulate(r->shape, fp, q, acc, st);
    launchAdvance(fp, r->dState, st);
    mark(7);
    return e;
}

int enqueuePass(optpt_renderer *r, const FrameParams &fp, cudaStream_t st, cudaEvent_t *ev, int *kind,
                bool count = false)
{
    return enqueuePassOn(r, fp, r->q, r->acc, st, ev, kind, count);
}

// Guiding buffers sized for the current frame (paths per pass, max depth),
// or for `minPaths` paths per pass if that is more (batched rendering).
int ensureGuideBuffers(optpt_renderer *r, size_t minPaths = 0, uint32_t stride = 0)
{
    if (r->guideMode == 0)
        return OPTPT_OK;
    const size_t paths = std::max((size_t)r->w * r->h * r->sppBatch, minPaths);
    stride = std::max(stride, r->gTrainStride);
    const size_t slots = ((paths + stride - 1) / stride) * std::max(1u, r->lp.maxDepth);
    if (r->gMix && r->gMixPaths >= paths && r->gRecSlots >= slots)
        return OPTPT_OK;
    r->freeGuideBuffers();
    cudaError_t e = cudaMalloc(&r->gMix, std::max<size_t>(paths, 1) * sizeof(guide::Packed));
    if (e == cudaSuccess)
        e = cudaMalloc(&r->gRec, std::max<size_t>(slots, 1) * GUIDE_REC * sizeof(float4));
    if (e == cudaSuccess)
        e = cudaMemset(r->gRec, 0, std::max<size_t>(slots, 1) * GUIDE_REC * sizeof(float4));
    if (e == cudaSuccess)
        e = cudaMalloc(&r->gBatch, (size_t)r->gBatchCap * sizeof(GuideSample));
    if (e == cudaSuccess)
        e = cudaMalloc(&r->gBatchCount, sizeof(uint32_t));
    if (e != cudaSuccess) {
        r->freeGuideBuffers();
        return fail(OPTPT_ERR_NOMEM, std::string("guiding buffers: ") + cudaGetErrorString(e));
    }
    r->gMixPaths = paths;
    r->gRecSlots = slots;
    r->graphDirty = true;
    r->batch.guideMode = -1;  // the batch graph holds the old pointers
    return OPTPT_OK;
}

int ensureGraph(optpt_renderer *r, cudaStream_t st)
{
    if (!r->graphDirty && r->graphExec)
        return OPTPT_OK;
    if (r->graphExec)
        cudaGraphExecDestroy(r->graphExec);
    if (r->graph)
        cudaGraphDestroy(r->graph);
    r->graphExec = nullptr;
    r->graph = nullptr;
    const FrameParams fp = r->frameParams();
    r->graphTrain = fp.guide.train != 0;
    CUDA_OR_RETURN(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    enqueuePass(r, fp, st, nullptr, nullptr);
    cudaError_t e = cudaStreamEndCapture(st, &r->graph);
    if (e != cudaSuccess)
        return cudaFail(e, "end capture");
    CUDA_OR_RETURN(cudaGraphInstantiate(&r->graphExec, r->graph, 0), "instantiate graph");
    r->graphDirty = false;
    return OPTPT_OK;
}

bool validScene(const optpt_scene *s, std::string &why)
{
    if (!s) {
        why = "scene is NULL";
        return false;
    }
    if (s->numTriangles && (!s->positions || !s->triIndices || !s->matIndices)) {
        why = "positions, triIndices and matIndices are required";
        return false;
    }
    if (s->numMaterials == 0 || !s->materials) {
        why = "at least one material is required";
        return false;
    }
    for (uint32_t t = 0; t < s->numTriangles; ++t) {
        for (int k = 0; k < 3; ++k) {
            int v = s->triIndices[3 * t + k];
            if (v < 0 || (uint32_t)v >= s->numVertices) {
                why = "triangle " + std::to_string(t) + " has a vertex index out of range";
                return false;
            }
        }
        int m = s->matIndices[t];
        if (m < 0 || (uint32_t)m >= s->numMaterials) {
            why = "triangle " + std::to_string(t) + " has a material index out of range";
            return false;
        }
    }
    for (uint32_t m = 0; m < s->numMaterials; ++m) {
        const int32_t *tex = &s->materials[m].baseColourTexture;
        for (int k = 0; k < 6; ++k) {
            if (tex[k] >= (int32_t)s->numTextures) {
                why = "material " + std::to_string(m) + " names a texture out of range";
                return false;
            }
        }
    }
    for (uint32_t t = 0; t < s->numTextures; ++t) {
        if (!s->textures[t].rgba || s->textures[t].width == 0 || s->textures[t].height == 0) {
            why = "texture " + std::to_string(t) + " is empty";
            return false;
        }
    }
    if (s->maxDepth > OPT_MAX_DEPTH) {
        why = "maxDepth above " + std::to_string(OPT_MAX_DEPTH);
        return false;
    }
    return true;
}

DevMaterial toDev(const MaterialData &m, uint32_t numTextures)
{
    DevMaterial d{};
    d.baseColour = make_float4(m.baseColour[0], m.baseColour[1], m.baseColour[2], m.baseColour[3]);
    d.emissionCutoff = make_float4(m.emission[0], m.emission[1], m.emission[2], m.alphaCutoff);
    d.sheen = make_float4(m.sheenColour[0], m.sheenColour[1], m.sheenColour[2], m.sheenRoughness);
    d.p0 = make_float4(m.ior, m.roughness, m.metallic, m.specular);
    d.p1 = make_float4(m.transmissionWeight, m.subsurfaceWeight, m.coatWeight, m.coatRoughness);
    const int32_t tex[6] = {m.baseColourTexture, m.normalTexture, m.metallicRoughnessTexture, m.emissiveTexture,
                            m.sheenColourTexture, m.sheenRoughnessTexture};
    const uint8_t has[6] = {m.hasBaseColourTexture, m.hasNormalTexture, m.hasMetallicRoughnessTexture,
                            m.hasEmissiveTexture, m.hasSheenColourTexture, m.hasSheenRoughnessTexture};
    const TextureTransform *tf[6] = {&m.baseColourTexTf, &m.normalTexTf, &m.metallicRoughnessTexTf,
                                     &m.emissiveTexTf, &m.sheenColourTexTf, &m.sheenRoughnessTexTf};
    int mask = 0;
    for (int k = 0; k < 6; ++k) {
        if (has[k] && tex[k] >= 0 && (uint32_t)tex[k] < numTextures)
            mask |= 1 << k;
        d.tf[k] = make_float4(tf[k]->offset[0], tf[k]->offset[1], tf[k]->scale[0], tf[k]->scale[1]);
    }
    d.flags = make_int4((int)m.category, m.alphaMode, mask, 0);
    d.tex0 = make_int4(tex[0], tex[1], tex[2], tex[3]);
    d.tex1 = make_int4(tex[4], tex[5], 0, 0);
    return d;
}

DevLight toDev(const Light &l)
{
    DevLight d{};
    int type = l.type;
    float tf;
    memcpy(&tf, &type, 4);
    d.p0Type = make_float4(l.p0[0], l.p0[1], l.p0[2], tf);
    d.radianceDist = make_float4(l.radiance[0], l.radiance[1], l.radiance[2], l.distance);
    d.normalCosW = make_float4(l.normal[0], l.normal[1], l.normal[2], l.cosWidth);
    d.cosFalloff = make_float4(l.cosFalloffStart, 0.0f, 0.0f, 0.0f);
    return d;
}

int checkRenderable(optpt_renderer *r)
{
    if (!r)
        return fail(OPTPT_ERR_INVALID, "renderer is NULL");
    if (r->w == 0 || r->h == 0)
        return fail(OPTPT_ERR_STATE, "no output buffer (call optpt_setup_output_buffer)");
    return OPTPT_OK;
}

}  // namespace

namespace {

// After the vertex positions changed (device arrays already updated on
// `st`): refit (BVH8) or rebuild (BVH2) the acceleration structure,
// regather the emissive-triangle vertices and restart accumulation, as
// Renderer::updateAccel does (buildAccel(false) then resetSampleCount,
// src/renderer.cpp:1299-1303).
int afterVertexChange(optpt_renderer *r, cudaStream_t st)
{
    const int nt = r->scene.numTris;
    if (r->bvh.nodes8) {
        int e = refitBvh8(r->bvh, r->dPositions, r->dTriIndices, nt, st);
        if (e)
            return cudaFail((cudaError_t)e, "BVH8 refit");
    } else if (nt > 0) {
        CUDA_OR_RETURN(cudaStreamSynchronize(st), "BVH rebuild");
        BvhBuild fresh{};
        int e = buildBvh(r->dPositions, r->dTriIndices, r->dMatIndices, r->dTriFlags, nt, (int)r->opt.leafSize, fresh,
                         st);
        if (e)
            return cudaFail((cudaError_t)e, "BVH rebuild");
        freeBvh(r->bvh);
        r->bvh = fresh;
        r->scene.nodes = r->bvh.nodes;
        r->scene.triV = r->bvh.triV;
        r->scene.numNodes = r->bvh.usedNodes;
        r->graphDirty = true;          // the captured pass holds the old pointers
        r->batch.guideMode = -1;
    }
    launchEmissiveVerts(r->numEmissive, r->dEmisPrim, r->dPositions, r->dTriIndices, nt, r->dEmisV, st);
    CUDA_OR_RETURN(cudaGetLastError(), "emissive vertices");
    if (r->w && r->h) {
        const size_t npix = (size_t)r->w * r->h;
        CUDA_OR_RETURN(cudaMemsetAsync(r->acc.sum, 0, sizeof(Acc4) * npix, st), "reset");
        CUDA_OR_RETURN(cudaMemsetAsync(r->acc.sumSq, 0, sizeof(Acc4) * npix, st), "reset");
        CUDA_OR_RETURN(cudaMemsetAsync(r->dState, 0, sizeof(uint32_t), st), "reset");
    }
    r->lp.sample = 0;
    r->hostFbValid = false;
    return OPTPT_OK;
}

template <class T> int replaceDevice(T *&dst, const T *src, size_t count, const char *what)
{
    cudaFree(dst);
    dst = nullptr;
    if (!src || !count)
        return OPTPT_OK;
    CUDA_OR_RETURN(cudaMalloc((void **)&dst, sizeof(T) * count), what);
    CUDA_OR_RETURN(cudaMemcpy(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice), what);
    return OPTPT_OK;
}

}  // namespace

extern "C" {

const char *optpt_last_error(void) { return g_lastError.c_str(); }

int optpt_internal_set_error(int code, const char *msg)
{
    g_lastError = msg ? msg : "";
    return code;
}

int optpt_version(void) { return 100; }

int optpt_create(const optpt_scene *s, const optpt_options *options, optpt_renderer **out)
{
    if (!out)
        return fail(OPTPT_ERR_INVALID, "out is NULL");
    *out = nullptr;
    std::string why;
    if (!validScene(s, why))
        return fail(OPTPT_ERR_INVALID, why);
    optpt_renderer *r = new (std::nothrow) optpt_renderer();
    if (!r)
        return fail(OPTPT_ERR_NOMEM, "host allocation failed");
    if (options)
        r->opt = *options;
    else
        r->opt.useGraph = 1;
    if (r->opt.bvhWidth == 0)
        r->opt.bvhWidth = 8;
    r->tailBounce = r->opt.tailBounce == 0 ? OPTPT_DEFAULT_TAIL_BOUNCE
                                           : (r->opt.tailBounce == 0xFFFFFFFFu ? 0u : r->opt.tailBounce);
    if (r->opt.bvhWidth != 2 && r->opt.bvhWidth != 8) {
        delete r;
        return fail(OPTPT_ERR_INVALID, "bvhWidth must be 2 or 8");
    }
    if (r->opt.compaction != 0 && r->opt.compaction != 1 && r->opt.compaction != 32) {
        delete r;
        return fail(OPTPT_ERR_INVALID, "compaction must be 0 (auto), 1 (per block) or 32 (per warp)");
    }
    if (r->opt.blockSize != 0 && (r->opt.blockSize % 32 != 0 || r->opt.blockSize > 256)) {
        delete r;
        return fail(OPTPT_ERR_INVALID, "blockSize must be a multiple of 32, at most 256");
    }
    if (r->opt.leafSize == 0)
        r->opt.leafSize = r->opt.bvhWidth == 8 ? 1 : 4;
    // BVH8 leaves address up to 32 triangles per node with 5-bit offsets.
    const uint32_t maxLeaf = r->opt.bvhWidth == 8 ? 4u : 8u;
    if (r->opt.leafSize > maxLeaf)
        r->opt.leafSize = maxLeaf;
    int rc = OPTPT_OK;
    cudaError_t e;
    do {
        if ((e = cudaStreamCreateWithFlags(&r->ownStream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaStreamCreateWithFlags(&r->sideStream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&r->evFork, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&r->evJoin, cudaEventDisableTiming)) != cudaSuccess) {
            rc = cudaFail(e, "stream");
            break;
        }
        if ((e = (cudaError_t)uploadSrgbTable()) != cudaSuccess) {
            rc = cudaFail(e, "sRGB table");
            break;
        }
        const uint32_t nt = s->numTriangles;
        r->numTris = (int)nt;
        for (int a = 0; a < 3; ++a) {
            r->sceneLo[a] = nt ? 3.4e38f : 0.0f;
            r->sceneHi[a] = nt ? -3.4e38f : 0.0f;
        }
        for (uint32_t v = 0; v < (nt ? s->numVertices : 0u); ++v)
            for (int a = 0; a < 3; ++a) {
                r->sceneLo[a] = std::min(r->sceneLo[a], s->positions[3 * v + a]);
                r->sceneHi[a] = std::max(r->sceneHi[a], s->positions[3 * v + a]);
            }
        std::vector<uint32_t> triFlags(nt);
        for (uint32_t t = 0; t < nt; ++t)
            triFlags[t] = s->materials[s->matIndices[t]].alphaMode != AM_OPAQUE ? TRI_FLAG_ALPHA : 0u;
        std::vector<DevMaterial> mats(s->numMaterials);
        for (uint32_t m = 0; m < s->numMaterials; ++m)
            mats[m] = toDev(s->materials[m], s->numTextures);
        std::vector<DevLight> lights(s->numLights);
        for (uint32_t l = 0; l < s->numLights; ++l)
            lights[l] = toDev(s->lights[l]);
        // Emissive triangles, in triangle order (src/gltf_loader.cpp:128-141,
        // src/renderer.cpp:210-237): emission > 0 or an emissive texture.
        std::vector<float4> emisV, emisRad;
        std::vector<float2> emisTc;
        std::vector<int> emisPrim;
        for (uint32_t t = 0; t < nt; ++t) {
            const MaterialData &m = s->materials[s->matIndices[t]];
            if (!(m.emission[0] > 0.0f || m.emission[1] > 0.0f || m.emission[2] > 0.0f || m.hasEmissiveTexture))
                continue;
            emisPrim.push_back((int)t);
            for (int k = 0; k < 3; ++k) {
                const int v = s->triIndices[3 * t + k];
                emisV.push_back(make_float4(s->positions[3 * v], s->positions[3 * v + 1], s->positions[3 * v + 2], 0.0f));
                emisTc.push_back(s->texCoords ? make_float2(s->texCoords[2 * v], s->texCoords[2 * v + 1])
                                              : make_float2(0.0f, 0.0f));
            }
            int mi = s->matIndices[t];
            float mf;
            memcpy(&mf, &mi, 4);
            emisRad.push_back(make_float4(m.emission[0], m.emission[1], m.emission[2], mf));
        }
        r->numEmissive = (int)emisRad.size();
        r->numLights = (int)s->numLights;
        r->numVerts = s->numVertices;
        r->hasNormals = s->normals != nullptr;
        std::vector<uint32_t> texels;
        std::vector<int4> texInfo;
        for (uint32_t t = 0; t < s->numTextures; ++t) {
            const optpt_texture &tx = s->textures[t];
            const int first = (int)texels.size();
            const size_t cnt = (size_t)tx.width * tx.height;
            texels.resize(texels.size() + cnt);
            memcpy(texels.data() + first, tx.rgba, cnt * 4);
            texInfo.push_back(make_int4(first, (int)tx.width, (int)tx.height,
                                        (tx.wrapS & 0xF) | ((tx.wrapT & 0xF) << 4) | ((tx.srgb ? 1 : 0) << 8) |
                                            ((tx.filter == 1 ? 1 : 0) << 9)));
        }
        if ((e = upload(r->dPositions, s->positions, (size_t)3 * s->numVertices)) ||
            (e = upload(r->dNormals, s->normals, s->normals ? (size_t)3 * s->numVertices : 0)) ||
            (e = upload(r->dTexCoords, s->texCoords, s->texCoords ? (size_t)2 * s->numVertices : 0)) ||
            (e = upload(r->dTriIndices, s->triIndices, (size_t)3 * nt)) ||
            (e = upload(r->dMatIndices, s->matIndices, (size_t)nt)) ||
            (e = upload(r->dTriFlags, triFlags.data(), triFlags.size())) ||
            (e = upload(r->dMaterials, mats.data(), mats.size())) ||
            (e = upload(r->dLights, lights.data(), lights.size())) ||
            (e = upload(r->dLightsPublic, s->lights, (size_t)s->numLights)) ||
            (e = upload(r->dEmisV, emisV.data(), emisV.size())) ||
            (e = upload(r->dEmisTc, emisTc.data(), emisTc.size())) ||
            (e = upload(r->dEmisRad, emisRad.data(), emisRad.size())) ||
            (e = upload(r->dEmisPrim, emisPrim.data(), emisPrim.size())) ||
            (e = upload(r->dTexels, texels.data(), texels.size())) ||
            (e = upload(r->dTexInfo, texInfo.data(), texInfo.size()))) {
            rc = cudaFail(e, "scene upload");
            break;
        }
        const bool ploc = r->opt.bvhWidth == 8 && r->opt.bvhBuilder == 1;
        int be = buildBvh(r->dPositions, r->dTriIndices, r->dMatIndices, r->dTriFlags, (int)nt, (int)r->opt.leafSize,
                          r->bvh, r->ownStream, ploc);
        if (be) {
            rc = cudaFail((cudaError_t)be, "BVH build");
            break;
        }
        if (r->opt.bvhWidth == 8 && (be = buildBvh8(r->bvh, (int)nt, r->ownStream))) {
            rc = cudaFail((cudaError_t)be, "BVH8 collapse");
            break;
        }
        if (ploc && r->bvh.nodes8 && r->bvh.levels8 > BVH8_STACK) {
            // A PLOC tree too deep for the traversal stack (clusters at
            // wildly different scales): the LBVH of the same order instead,
            // whose depth the Morton bits bound.
            freeBvh(r->bvh);
            if ((be = buildBvh(r->dPositions, r->dTriIndices, r->dMatIndices, r->dTriFlags, (int)nt,
                               (int)r->opt.leafSize, r->bvh, r->ownStream, false)) ||
                (be = buildBvh8(r->bvh, (int)nt, r->ownStream))) {
                rc = cudaFail((cudaError_t)be, "BVH build");
                break;
            }
        }
        // A ray's node-group stack holds at most one group per level below
        // the root: a tree of at most BVH8_STACK levels cannot overflow it.
        if (r->bvh.nodes8 && r->bvh.levels8 > BVH8_STACK) {
            rc = fail(OPTPT_ERR_INVALID, "BVH8 of " + std::to_string(r->bvh.levels8) + " levels exceeds the " +
                                             std::to_string(BVH8_STACK) + "-entry traversal stack");
            break;
        }
        DevScene &ds = r->scene;
        ds.nodes = r->bvh.nodes;
        ds.nodes8 = r->bvh.nodes8;
        ds.triV = r->bvh.nodes8 ? r->bvh.triV8 : r->bvh.triV;
        ds.triIndices = r->dTriIndices;
        ds.normals = r->dNormals;
        ds.texCoords = r->dTexCoords;
        ds.materials = r->dMaterials;
        ds.lights = r->dLights;
        ds.emisV = r->dEmisV;
        ds.emisTc = r->dEmisTc;
        ds.emisRad = r->dEmisRad;
        ds.texels = r->dTexels;
        ds.texInfo = r->dTexInfo;
        ds.numNodes = r->bvh.usedNodes;
        ds.numTris = (int)nt;
        ds.numLights = r->numLights;
        ds.numEmissive = r->numEmissive;
        ds.nodeBudget = r->opt.nodeBudget ? (int)std::min<uint32_t>(r->opt.nodeBudget, INT_MAX) : TRAV_DEFAULT_BUDGET;
        if ((e = cudaMalloc((void **)&r->q.counters, sizeof(uint32_t) * CNT_TOTAL)) ||
            (e = cudaMalloc((void **)&r->q.totals, sizeof(unsigned long long) * TOTALS_COUNT)) ||
            (e = cudaMemset(r->q.totals, 0, sizeof(unsigned long long) * TOTALS_COUNT)) ||
            (e = cudaMalloc((void **)&r->dState, sizeof(uint32_t) * 4)) ||
            (e = cudaMemset(r->dState, 0, sizeof(uint32_t) * 4)) ||
            (e = cudaMalloc((void **)&r->dFrameConst, sizeof(FrameConst))) ||
            (e = cudaHostAlloc((void **)&r->hFrameConst, sizeof(FrameConst) * optpt_renderer::FC_SLOTS,
                               cudaHostAllocDefault))) {
            rc = cudaFail(e, "counters");
            break;
        }
        for (auto &ev : r->fcCopied)
            if (!e)
                e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e) {
            rc = cudaFail(e, "events");
            break;
        }
        // Frame contract defaults (src/renderer.cpp:24-60, include/renderer.h:137-146).
        LaunchParams &lp = r->lp;
        lp.seed = 1;
        lp.traversable = (uint64_t)(uintptr_t)r->bvh.nodes;
        lp.lights = r->dLightsPublic;
        lp.numLights = s->numLights;
        lp.numEmissiveTriangles = (uint32_t)r->numEmissive;
        lp.randState = nullptr;
        lp.vis = 0;
        lp.toneMapping = 1;
        lp.toneMappingImpl = 1;
        lp.gammaCorrection = 1;
        lp.gammaTerm = 2.2f;
        lp.maxDepth = s->maxDepth ? s->maxDepth : 8;
        memcpy(lp.bgColour, s->bgColour, sizeof(lp.bgColour));
        rc = allocFrame(r, s->resX ? s->resX : 512, s->resY ? s->resY : 512);
        if (rc)
            break;
        const float aspect = (float)r->w / (float)r->h;
        cameraBasis(s->camEye, s->camTarget, s->camUp, s->camFovYDeg > 0 ? s->camFovYDeg : 40.0f, aspect, lp.U, lp.V,
                    lp.W);
        memcpy(lp.eye, s->camEye, sizeof(lp.eye));
    } while (0);
    if (rc != OPTPT_OK) {
        delete r;
        return rc;
    }
    *out = r;
    return OPTPT_OK;
}

}  // extern "C"

namespace {

// Batched multi-view rendering, step 1: checks the views, (re)allocates the
// batch buffers for their pixel layout, restarts the accumulators and
// captures the batch pass (once per layout and guiding mode).
int batchSetup(optpt_renderer *r, const optpt_view *views, uint32_t numViews, cudaStream_t st)
{
    if (!r || (numViews && !views))
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if (numViews == 0 || numViews > 65535)
        return fail(OPTPT_ERR_INVALID, "between 1 and 65535 views");
    uint64_t total = 0;
    for (uint32_t v = 0; v < numViews; ++v) {
        const optpt_view &V = views[v];
        if (V.width == 0 || V.height == 0 || V.spp == 0 || !(V.fovYDeg > 0.0f && V.fovYDeg < 180.0f))
            return fail(OPTPT_ERR_INVALID, "view " + std::to_string(v) + ": width, height, spp > 0, fovYDeg in (0, 180)");
        total += (uint64_t)V.width * V.height;
    }
    if (total > (1u << 30))
        return fail(OPTPT_ERR_INVALID, "more than 2^30 pixels in one batch");
    auto &B = r->batch;
    if (r->shape.block == 0) {
        const int blk = r->opt.blockSize ? (int)r->opt.blockSize : 128;
        r->shape.block = blk;
        r->shape.compaction = r->opt.compaction == 1 ? 1 : 0;
        r->shape.gridGenerate = occupancyGrid(0, blk);
        const bool wide = r->bvh.nodes8 != nullptr;
        r->shape.gridExtend = occupancyGrid(wide ? 1 : 11, blk);
        r->shape.gridShade = occupancyGrid(2, blk);
        r->shape.gridShadow = occupancyGrid(wide ? 3 : 13, blk);
        r->shape.gridAccum = occupancyGrid(4, blk);
        r->shape.gridFinish = occupancyGrid(wide ? 5 : 15, 128);
    }
    // (Re)allocate when the pixel layout changes; paths per pass: at least one
    // sample for every pixel, and about 2^21 paths when fewer pixels are active.
    bool layout = B.views.size() != numViews || B.maxDepth != r->lp.maxDepth;
    for (uint32_t v = 0; !layout && v < numViews; ++v)
        layout = B.views[v].width != views[v].width || B.views[v].height != views[v].height;
    if (layout) {
        r->freeBatch();
        B.totalPixels = (uint32_t)total;
        B.maxPaths = std::max<uint32_t>(B.totalPixels, 1u << 21);
        B.maxDepth = r->lp.maxDepth;
        const size_t P = B.maxPaths, N = B.totalPixels;
        cudaError_t e = cudaSuccess;
        auto al = [&](void **p, size_t bytes) {
            if (e == cudaSuccess)
                e = cudaMalloc(p, bytes ? bytes : 16);
        };
        float4 **bufs[] = {&B.q.pathT, &B.q.pathL, &B.q.rayO[0], &B.q.rayO[1], &B.q.rayD[0], &B.q.rayD[1], &B.q.hit,
                           &B.q.shO[0], &B.q.shO[1], &B.q.shD[0], &B.q.shD[1], &B.q.shC[0], &B.q.shC[1]};
        for (float4 **b : bufs)
            al((void **)b, sizeof(float4) * P);
        al((void **)&B.acc.sum, sizeof(Acc4) * N);
        al((void **)&B.acc.sumSq, sizeof(Acc4) * N);
        al((void **)&B.acc.frameBuffer, sizeof(float4) * N);
        al((void **)&B.acc.accumFrameBuffer, sizeof(float4) * N);
        al((void **)&B.dViews, sizeof(BatchView) * numViews);
        al((void **)&B.dPixelList, sizeof(uint32_t) * N);
        al((void **)&B.dPixelView, sizeof(uint16_t) * N);
        al((void **)&B.dDyn, sizeof(uint32_t) * 2);
        if (e != cudaSuccess) {
            r->freeBatch();
            return fail(OPTPT_ERR_NOMEM, std::string("batch buffers: ") + cudaGetErrorString(e));
        }
        B.views.assign(views, views + numViews);
        B.first.resize(numViews);
        std::vector<uint16_t> pv(N);
        uint32_t at = 0;
        for (uint32_t v = 0; v < numViews; ++v) {
            B.first[v] = at;
            const uint32_t n = views[v].width * views[v].height;
            std::fill(pv.begin() + at, pv.begin() + at + n, (uint16_t)v);
            at += n;
        }
        CUDA_OR_RETURN(cudaMemcpy(B.dPixelView, pv.data(), sizeof(uint16_t) * N, cudaMemcpyHostToDevice), "batch");
    }
    B.views.assign(views, views + numViews);
    B.q.counters = r->q.counters;
    B.q.totals = r->q.totals;
    // large batches record one training path in `stride` (about 2^21 per pass)
    const uint32_t stride = std::max(r->gTrainStride, (B.maxPaths + (1u << 21) - 1) >> 21);
    int rc = ensureGuideBuffers(r, B.maxPaths, stride);
    if (rc)
        return rc;
    CUDA_OR_RETURN(cudaMemsetAsync(B.acc.sum, 0, sizeof(Acc4) * B.totalPixels, st), "batch");
    CUDA_OR_RETURN(cudaMemsetAsync(B.acc.sumSq, 0, sizeof(Acc4) * B.totalPixels, st), "batch");
    B.done.assign(numViews, 0u);
    CUDA_OR_RETURN(r->uploadFrameConst(st), "frame constants");

    FrameParams fp = r->frameParams();
    fp.w = fp.h = fp.npix = fp.sppBatch = 0;
    fp.numPaths = B.maxPaths;
    fp.batch = BatchPass{B.dViews, B.dPixelList, B.dPixelView, B.dDyn, 1u};
    if (fp.guide.on) {  // the guiding buffers now hold the batch's paths
        fp.guide.mix = r->gMix;
        fp.guide.rec = r->gRec;
        fp.guide.trainStride = stride;
    }
    // one captured pass; every replay reads its sizes from the device
    if (!B.exec || B.guideMode != r->guideMode || r->graphDirty) {
        if (B.exec)
            cudaGraphExecDestroy(B.exec);
        if (B.graph)
            cudaGraphDestroy(B.graph);
        B.exec = nullptr;
        B.graph = nullptr;
        cudaStream_t cs = st ? st : r->ownStream;
        CUDA_OR_RETURN(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "batch capture");
        enqueuePassOn(r, fp, B.q, B.acc, cs, nullptr, nullptr);
        cudaError_t e = cudaStreamEndCapture(cs, &B.graph);
        if (e != cudaSuccess)
            return cudaFail(e, "batch capture");
        CUDA_OR_RETURN(cudaGraphInstantiate(&B.exec, B.graph, 0), "batch instantiate");
        B.guideMode = r->guideMode;
    }
    B.wasActive.assign(numViews, 0);
    B.list.clear();
    B.per = 0;
    return OPTPT_OK;
}

// Step 2, once per pass: picks the views that still need samples and the
// samples per pixel of this pass, and uploads the active-pixel list (when it
// changed), the view table and the pass sizes on `st`. *more = false when
// every view is done (nothing is uploaded then).
int batchPassSizes(optpt_renderer *r, cudaStream_t st, bool *more)
{
    auto &B = r->batch;
    const std::vector<optpt_view> &views = B.views;
    const uint32_t numViews = (uint32_t)views.size();
    uint32_t active = 0, minLeft = UINT32_MAX;
    bool changed = false;
    for (uint32_t v = 0; v < numViews; ++v) {
        const bool a = B.done[v] < views[v].spp;
        changed |= (a != (bool)B.wasActive[v]);
        B.wasActive[v] = a;
        if (a) {
            active += views[v].width * views[v].height;
            minLeft = std::min(minLeft, views[v].spp - B.done[v]);
        }
    }
    *more = active != 0;
    if (!*more)
        return OPTPT_OK;
    if (changed) {
        B.list.clear();
        for (uint32_t v = 0; v < numViews; ++v)
            if (B.wasActive[v])
                for (uint32_t k = 0; k < views[v].width * views[v].height; ++k)
                    B.list.push_back(B.first[v] + k);
        CUDA_OR_RETURN(cudaMemcpyAsync(B.dPixelList, B.list.data(), sizeof(uint32_t) * B.list.size(),
                                       cudaMemcpyHostToDevice, st),
                       "batch list");
    }
    B.per = std::max(1u, std::min(minLeft, B.maxPaths / active));
    B.hostViews.resize(numViews);
    for (uint32_t v = 0; v < numViews; ++v) {
        const optpt_view &V = views[v];
        float U[3], Vv[3], W[3];
        cameraBasis(V.eye, V.target, V.up, V.fovYDeg, (float)V.width / (float)V.height, U, Vv, W);
        auto bits = [](uint32_t u) {
            float f;
            memcpy(&f, &u, 4);
            return f;
        };
        B.hostViews[v].eye = make_float4(V.eye[0], V.eye[1], V.eye[2], bits(V.width));
        B.hostViews[v].U = make_float4(U[0], U[1], U[2], bits(V.height));
        B.hostViews[v].V = make_float4(Vv[0], Vv[1], Vv[2], bits(B.first[v]));
        B.hostViews[v].W = make_float4(W[0], W[1], W[2], bits(B.done[v]));
    }
    B.dyn[0] = active;
    B.dyn[1] = B.per;
    CUDA_OR_RETURN(cudaMemcpyAsync(B.dViews, B.hostViews.data(), sizeof(BatchView) * numViews,
                                   cudaMemcpyHostToDevice, st),
                   "batch views");
    CUDA_OR_RETURN(cudaMemcpyAsync(B.dDyn, B.dyn, sizeof(B.dyn), cudaMemcpyHostToDevice, st), "batch sizes");
    return OPTPT_OK;
}

// Step 3, after the pass is enqueued: the active views' sample counts.
void batchPassDone(optpt_renderer *r)
{
    auto &B = r->batch;
    for (size_t v = 0; v < B.views.size(); ++v)
        if (B.wasActive[v])
            B.done[v] += B.per;
}

}  // namespace

extern "C" {

int optpt_render_batch(optpt_renderer *r, const optpt_view *views, uint32_t numViews, void *stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    int rc = batchSetup(r, views, numViews, st);
    if (rc)
        return rc;
    for (;;) {
        bool more = false;
        if ((rc = batchPassSizes(r, st, &more)))
            return rc;
        if (!more)
            break;
        CUDA_OR_RETURN(cudaGraphLaunch(r->batch.exec, st), "batch launch");
        batchPassDone(r);
    }
    CUDA_OR_RETURN(cudaGetLastError(), "batch");
    return OPTPT_OK;
}

int optpt_render_batch_scenes(optpt_renderer *const *renderers, uint32_t numScenes, const optpt_view *views,
                              uint32_t numViews, void *stream)
{
    if (!renderers || numScenes == 0 || numScenes > 32 || !views || numViews == 0)
        return fail(OPTPT_ERR_INVALID, "1 to 32 renderers and at least one view");
    for (uint32_t k = 0; k < numScenes; ++k) {
        if (!renderers[k])
            return fail(OPTPT_ERR_INVALID, "NULL renderer");
        for (uint32_t j = 0; j < k; ++j)
            if (renderers[j] == renderers[k])
                return fail(OPTPT_ERR_INVALID, "a renderer appears twice (one renderer per scene)");
    }
    std::vector<std::vector<optpt_view>> per(numScenes);
    for (uint32_t v = 0; v < numViews; ++v) {
        if (views[v].scene >= numScenes)
            return fail(OPTPT_ERR_INVALID, "view " + std::to_string(v) + ": scene index out of range");
        per[views[v].scene].push_back(views[v]);
    }
    cudaStream_t st = (cudaStream_t)stream;
    int rc;
    for (uint32_t k = 0; k < numScenes; ++k)
        if (!per[k].empty() && (rc = batchSetup(renderers[k], per[k].data(), (uint32_t)per[k].size(), st)))
            return rc;
    // One graph per set of still-active scenes: each scene's captured batch
    // pass is a child graph, with no dependency between them, so one launch
    // runs every scene's pass and their bounce loops proceed side by side.
    std::vector<std::pair<uint32_t, cudaGraphExec_t>> execs;
    std::vector<cudaGraph_t> graphs;
    auto cleanup = [&]() {
        for (auto &e : execs)
            cudaGraphExecDestroy(e.second);
        for (cudaGraph_t g : graphs)
            cudaGraphDestroy(g);
    };
    for (;;) {
        uint32_t mask = 0;
        for (uint32_t k = 0; k < numScenes; ++k) {
            if (per[k].empty())
                continue;
            bool more = false;
            if ((rc = batchPassSizes(renderers[k], st, &more))) {
                cleanup();
                return rc;
            }
            if (more)
                mask |= 1u << k;
        }
        if (mask == 0)
            break;
        cudaGraphExec_t exec = nullptr;
        for (auto &e : execs)
            if (e.first == mask)
                exec = e.second;
        if (!exec) {
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaGraphCreate(&g, 0);
            for (uint32_t k = 0; e == cudaSuccess && k < numScenes; ++k) {
                cudaGraphNode_t node;
                if (mask & (1u << k))
                    e = cudaGraphAddChildGraphNode(&node, g, nullptr, 0, renderers[k]->batch.graph);
            }
            if (e == cudaSuccess)
                e = cudaGraphInstantiate(&exec, g, 0);
            if (g)
                graphs.push_back(g);
            if (e != cudaSuccess) {
                cleanup();
                return cudaFail(e, "multi-scene batch graph");
            }
            execs.emplace_back(mask, exec);
        }
        cudaError_t e = cudaGraphLaunch(exec, st);
        if (e != cudaSuccess) {
            cleanup();
            return cudaFail(e, "multi-scene batch launch");
        }
        for (uint32_t k = 0; k < numScenes; ++k)
            if (mask & (1u << k))
                batchPassDone(renderers[k]);
    }
    // the graphs may be destroyed once their launches are enqueued
    cleanup();
    CUDA_OR_RETURN(cudaGetLastError(), "multi-scene batch");
    return OPTPT_OK;
}

int optpt_batch_view(optpt_renderer *r, uint32_t view, double **sum, double **sumSq, float **frameBuffer,
                     uint32_t *samples)
{
    if (!r)
        return fail(OPTPT_ERR_INVALID, "NULL renderer");
    if (view >= r->batch.views.size())
        return fail(OPTPT_ERR_INVALID, "no such view in the last batch");
    const uint32_t f = r->batch.first[view];
    if (sum)
        *sum = reinterpret_cast<double *>(r->batch.acc.sum + f);
    if (sumSq)
        *sumSq = reinterpret_cast<double *>(r->batch.acc.sumSq + f);
    if (frameBuffer)
        *frameBuffer = reinterpret_cast<float *>(r->batch.acc.frameBuffer + f);
    if (samples)
        *samples = r->batch.done.empty() ? 0u : r->batch.done[view];
    return OPTPT_OK;
}

int optpt_batch_read_view(optpt_renderer *r, uint32_t view, double *sumHost, double *sumSqHost, void *stream)
{
    double *s = nullptr, *q = nullptr;
    int rc = optpt_batch_view(r, view, &s, &q, nullptr, nullptr);
    if (rc)
        return rc;
    const size_t n = (size_t)r->batch.views[view].width * r->batch.views[view].height;
    cudaStream_t st = (cudaStream_t)stream;
    if (sumHost)
        CUDA_OR_RETURN(cudaMemcpyAsync(sumHost, s, sizeof(Acc4) * n, cudaMemcpyDeviceToHost, st), "read view");
    if (sumSqHost)
        CUDA_OR_RETURN(cudaMemcpyAsync(sumSqHost, q, sizeof(Acc4) * n, cudaMemcpyDeviceToHost, st), "read view");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "read view");
    return OPTPT_OK;
}

int optpt_set_guiding(optpt_renderer *r, int mode)
{
    if (!r)
        return fail(OPTPT_ERR_INVALID, "NULL renderer");
    if (mode < 0 || mode > 2)
        return fail(OPTPT_ERR_INVALID, "guiding mode must be 0 (off), 1 (guided, training) or 2 (guided, frozen)");
    if (mode != 0 && !r->guide) {
        optpt_guide *g = new optpt_guide();
        int rc = guideCreate(g, r->sceneLo, r->sceneHi, r->lp.seed);
        if (rc != OPTPT_OK) {
            delete g;
            return rc;
        }
        g->lr = r->gLr;
        g->lobeLoss = r->gLobeLoss;
        r->guide = g;
        r->gTrainedSpp = 0;
    }
    if (mode != r->guideMode) {
        r->guideMode = mode;
        r->graphDirty = true;
    }
    return ensureGuideBuffers(r);
}

int optpt_set_guiding_options(optpt_renderer *r, const optpt_guiding_options *o)
{
    if (!r || !o)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if (o->alphaMax < 0.0f || o->alphaMax >= 1.0f || o->alphaMin < 0.0f || o->alphaMin >= 1.0f ||
        o->alphaRamp < 0.0f || o->learningRate < 0.0f || o->lobeLoss < 0 || o->lobeLoss > 2)
        return fail(OPTPT_ERR_INVALID, "alphaMin, alphaMax must lie in [0, 1); alphaRamp, learningRate >= 0; "
                                       "lobeLoss 0, 1 or 2");
    if (o->alphaMin > 0.0f)
        r->gAlphaMin = o->alphaMin;
    if (o->lobeLoss) {
        r->gLobeLoss = o->lobeLoss - 1;
        if (r->guide)
            r->guide->lobeLoss = r->gLobeLoss;
    }
    if (o->trainSteps > 64)
        return fail(OPTPT_ERR_INVALID, "at most 64 training steps per pass");
    if (o->trainSteps)
        r->gTrainSteps = o->trainSteps;
    if (o->trainStride)
        r->gTrainStride = o->trainStride;
    if (o->maxDepth)
        r->gMaxDepth = o->maxDepth;
    if (o->primaryShare)
        r->gSharePrimary = o->primaryShare > 0;
    if (o->trainSpp && o->trainSpp != r->gTrainSpp) {
        r->gTrainSpp = o->trainSpp;
        r->gTrainedSpp = 0;  // a new budget starts now
    }
    if (o->alphaMax > 0.0f)
        r->gAlphaMax = o->alphaMax;
    if (o->alphaRamp > 0.0f)
        r->gAlphaRamp = o->alphaRamp;
    if (o->learningRate > 0.0f) {
        r->gLr = o->learningRate;
        if (r->guide)
            r->guide->lr = o->learningRate;
    }
    r->graphDirty = true;
    return ensureGuideBuffers(r);
}

int optpt_get_guiding_options(const optpt_renderer *r, optpt_guiding_options *o)
{
    if (!r || !o)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    o->trainSteps = r->gTrainSteps;
    o->trainStride = r->gTrainStride;
    o->maxDepth = r->gMaxDepth;
    o->trainSpp = r->gTrainSpp;
    o->primaryShare = r->gSharePrimary ? 1 : -1;
    o->alphaMin = r->gAlphaMin;
    o->alphaMax = r->gAlphaMax;
    o->lobeLoss = r->gLobeLoss + 1;
    o->alphaRamp = r->gAlphaRamp;
    o->learningRate = r->gLr;
    return OPTPT_OK;
}

int optpt_guiding_batch(optpt_renderer *r, float *samples, uint32_t capacity, uint32_t *count)
{
    if (!r || !count)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    *count = 0;
    if (!r->gBatchCount)
        return OPTPT_OK;
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "guiding batch");
    uint32_t n = 0;
    CUDA_OR_RETURN(cudaMemcpy(&n, r->gBatchCount, sizeof(n), cudaMemcpyDeviceToHost), "guiding batch");
    n = std::min(n, r->gBatchCap);
    *count = n;
    if (samples && capacity)
        CUDA_OR_RETURN(cudaMemcpy(samples, r->gBatch, sizeof(GuideSample) * std::min(n, capacity),
                                  cudaMemcpyDeviceToHost),
                       "guiding batch");
    return OPTPT_OK;
}

int optpt_queue_counts(optpt_renderer *r, uint32_t *ext, uint32_t *shadowPoint, uint32_t *shadowEmissive,
                       uint32_t maxDepth)
{
    if (!r)
        return fail(OPTPT_ERR_INVALID, "NULL renderer");
    if (maxDepth > OPT_MAX_DEPTH)
        return fail(OPTPT_ERR_INVALID, "maxDepth out of range");
    uint32_t c[CNT_TOTAL];
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "queue counts");
    CUDA_OR_RETURN(cudaMemcpy(c, r->q.counters, sizeof(c), cudaMemcpyDeviceToHost), "queue counts");
    for (uint32_t d = 1; d <= maxDepth; ++d) {
        if (ext)
            ext[d - 1] = c[CNT_EXT + d];
        if (shadowPoint)
            shadowPoint[d - 1] = c[CNT_SHADOW_P + d];
        if (shadowEmissive)
            shadowEmissive[d - 1] = c[CNT_SHADOW_E + d];
    }
    return OPTPT_OK;
}

int optpt_get_guide(optpt_renderer *r, optpt_guide **out)
{
    if (!r || !out)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    *out = r->guide;
    return OPTPT_OK;
}

int optpt_destroy(optpt_renderer *r)
{
    if (!r)
        return OPTPT_OK;
    cudaDeviceSynchronize();
    delete r;
    return OPTPT_OK;
}

int optpt_setup_output_buffer(optpt_renderer *r, uint32_t width, uint32_t height)
{
    if (!r)
        return fail(OPTPT_ERR_INVALID, "renderer is NULL");
    if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 27))
        return fail(OPTPT_ERR_INVALID, "output size out of range");
    cudaDeviceSynchronize();
    return allocFrame(r, width, height);
}

int optpt_setup_camera(optpt_renderer *r, const float eye[3], const float target[3], const float up[3],
                       float fovYDeg)
{
    if (!r || !eye || !target || !up)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if (!(fovYDeg > 0.0f && fovYDeg < 180.0f))
        return fail(OPTPT_ERR_INVALID, "fovYDeg out of range");
    const float aspect = r->h ? (float)r->w / (float)r->h : 1.0f;
    cameraBasis(eye, target, up, fovYDeg, aspect, r->lp.U, r->lp.V, r->lp.W);
    memcpy(r->lp.eye, eye, sizeof(r->lp.eye));
    return OPTPT_OK;
}

int optpt_get_launch_params(const optpt_renderer *r, LaunchParams *out)
{
    if (!r || !out)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    *out = r->lp;
    return OPTPT_OK;
}

int optpt_set_launch_params(optpt_renderer *r, const LaunchParams *lp)
{
    if (!r || !lp)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if (lp->maxDepth < 1 || lp->maxDepth > OPT_MAX_DEPTH)
        return fail(OPTPT_ERR_INVALID, "maxDepth out of range");
    if (lp->toneMappingImpl != 0 && lp->toneMappingImpl != 1)
        return fail(OPTPT_ERR_INVALID, "toneMappingImpl must be 0 or 1");
    if (lp->sample != r->lp.sample) {
        const uint32_t st = lp->sample;  // state[1] (the pass count) runs on
        CUDA_OR_RETURN(cudaDeviceSynchronize(), "set sample");
        CUDA_OR_RETURN(cudaMemcpy(r->dState, &st, sizeof(st), cudaMemcpyHostToDevice), "set sample");
    }
    if (lp->maxDepth != r->lp.maxDepth)
        r->graphDirty = true;
    LaunchParams &d = r->lp;
    d.sample = lp->sample;
    d.seed = lp->seed;
    memcpy(d.eye, lp->eye, sizeof(d.eye));
    memcpy(d.U, lp->U, sizeof(d.U));
    memcpy(d.V, lp->V, sizeof(d.V));
    memcpy(d.W, lp->W, sizeof(d.W));
    d.vis = lp->vis;
    d.toneMapping = lp->toneMapping;
    d.toneMappingImpl = lp->toneMappingImpl;
    d.gammaCorrection = lp->gammaCorrection;
    d.gammaTerm = lp->gammaTerm;
    d.maxDepth = lp->maxDepth;
    memcpy(d.bgColour, lp->bgColour, sizeof(d.bgColour));
    return OPTPT_OK;
}

int optpt_render(optpt_renderer *r, uint32_t spp, void *stream)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // The frame constants go up first (from the pinned ring, so the host
    // copy may change as soon as this returns). Whole passes of sppBatch
    // samples replay the captured graph; a remainder runs as one smaller pass.
    CUDA_OR_RETURN(r->uploadFrameConst(st), "frame constants");
    if ((rc = ensureGuideBuffers(r)))
        return rc;
    const uint32_t passes = spp / r->sppBatch, rem = spp % r->sppBatch;
    // Online training runs until its sample budget is spent; the pass after
    // that is recaptured without it (the network is then frozen).
    for (uint32_t p = 0; p < passes; ++p) {
        const bool training = r->trainingOpen();
        if (r->opt.useGraph) {
            if (training != r->graphTrain)
                r->graphDirty = true;
            if ((rc = ensureGraph(r, st ? st : r->ownStream)))
                return rc;
            CUDA_OR_RETURN(cudaGraphLaunch(r->graphExec, st), "graph launch");
        } else {
            enqueuePass(r, r->frameParams(), st, nullptr, nullptr);
        }
        if (training)
            r->gTrainedSpp += r->sppBatch;
    }
    if (rem) {
        const bool training = r->trainingOpen();
        FrameParams fp = r->frameParams();
        fp.sppBatch = rem;
        fp.numPaths = r->w * r->h * rem;
        enqueuePass(r, fp, st, nullptr, nullptr);
        if (training)
            r->gTrainedSpp += rem;
    }
    CUDA_OR_RETURN(cudaGetLastError(), "kernel launch");
    r->lp.sample += spp;
    r->hostFbValid = false;
    return OPTPT_OK;
}

int optpt_launch(optpt_renderer *r)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if ((rc = optpt_render(r, 1, r->ownStream)))
        return rc;
    CUDA_OR_RETURN(cudaMemcpyAsync(r->hostFb.data(), r->acc.frameBuffer, sizeof(float4) * r->w * r->h,
                                   cudaMemcpyDeviceToHost, r->ownStream),
                   "frame buffer copy");
    CUDA_OR_RETURN(cudaStreamSynchronize(r->ownStream), "launch");
    r->hostFbValid = true;
    return OPTPT_OK;
}

int optpt_launch_pipelined(optpt_renderer *r, const float **frame)
{
    if (frame)
        *frame = nullptr;
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (!frame)
        return fail(OPTPT_ERR_INVALID, "frame is NULL");
    auto &P = r->pipe;
    const size_t npix = (size_t)r->w * r->h, bytes = sizeof(float4) * npix;
    if (P.pixels != npix) {
        r->freePipe();
        cudaError_t e = cudaStreamCreateWithFlags(&P.copyStream, cudaStreamNonBlocking);
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
            e = cudaMalloc((void **)&P.stage[k], bytes);
            if (e == cudaSuccess)
                e = cudaHostAlloc((void **)&P.host[k], bytes, cudaHostAllocDefault);
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&P.staged[k], cudaEventDisableTiming);
            if (e == cudaSuccess)
                e = cudaEventCreateWithFlags(&P.copied[k], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            r->freePipe();
            return cudaFail(e, "pipelined frame buffers");
        }
        P.pixels = npix;
    }
    const uint32_t k = P.next;
    if ((rc = optpt_render(r, 1, r->ownStream)))
        return rc;
    // The snapshot reuses slot k: the copy made from it two frames ago must
    // have finished (a wait on an event never recorded returns at once).
    CUDA_OR_RETURN(cudaStreamWaitEvent(r->ownStream, P.copied[k], 0), "pipelined launch");
    launchCopyFrame(r->acc.frameBuffer, P.stage[k], npix, r->ownStream);
    CUDA_OR_RETURN(cudaGetLastError(), "frame snapshot");
    CUDA_OR_RETURN(cudaEventRecord(P.staged[k], r->ownStream), "pipelined launch");
    CUDA_OR_RETURN(cudaStreamWaitEvent(P.copyStream, P.staged[k], 0), "pipelined launch");
    CUDA_OR_RETURN(cudaMemcpyAsync(P.host[k], P.stage[k], bytes, cudaMemcpyDeviceToHost, P.copyStream),
                   "frame copy");
    CUDA_OR_RETURN(cudaEventRecord(P.copied[k], P.copyStream), "pipelined launch");
    const int prev = P.pending;
    P.pending = (int)k;
    P.next = k ^ 1u;
    if (prev >= 0) {
        CUDA_OR_RETURN(cudaEventSynchronize(P.copied[prev]), "frame copy");
        *frame = P.host[prev];
    }
    return OPTPT_OK;
}

int optpt_launch_flush(optpt_renderer *r, const float **frame)
{
    if (frame)
        *frame = nullptr;
    if (!r || !frame)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    auto &P = r->pipe;
    if (P.pending < 0)
        return OPTPT_OK;
    const int k = P.pending;
    P.pending = -1;
    CUDA_OR_RETURN(cudaEventSynchronize(P.copied[k]), "frame copy");
    *frame = P.host[k];
    return OPTPT_OK;
}

const float *optpt_get_frame_buffer(optpt_renderer *r)
{
    if (!r || !r->hostFbValid)
        return nullptr;
    return r->hostFb.data();
}

uint32_t optpt_get_sample_count(const optpt_renderer *r) { return r ? r->lp.sample : 0u; }

int optpt_reset_sample_count(optpt_renderer *r)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    cudaDeviceSynchronize();
    const size_t npix = (size_t)r->w * r->h;
    CUDA_OR_RETURN(cudaMemset(r->acc.sum, 0, sizeof(Acc4) * npix), "reset");
    CUDA_OR_RETURN(cudaMemset(r->acc.sumSq, 0, sizeof(Acc4) * npix), "reset");
    CUDA_OR_RETURN(cudaMemset(r->dState, 0, sizeof(uint32_t)), "reset");
    r->lp.sample = 0;
    r->hostFbValid = false;
    return OPTPT_OK;
}

int optpt_device_buffers(optpt_renderer *r, float **frameBuffer, float **accumFrameBuffer, double **sum,
                         double **sumSq)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (frameBuffer)
        *frameBuffer = (float *)r->acc.frameBuffer;
    if (accumFrameBuffer)
        *accumFrameBuffer = (float *)r->acc.accumFrameBuffer;
    if (sum)
        *sum = (double *)r->acc.sum;
    if (sumSq)
        *sumSq = (double *)r->acc.sumSq;
    return OPTPT_OK;
}

int optpt_read_frame_buffer(optpt_renderer *r, float *rgbaHost, void *stream)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (!rgbaHost)
        return fail(OPTPT_ERR_INVALID, "NULL destination");
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_OR_RETURN(cudaMemcpyAsync(rgbaHost, r->acc.frameBuffer, sizeof(float4) * r->w * r->h,
                                   cudaMemcpyDeviceToHost, st),
                   "frame buffer copy");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "frame buffer copy");
    return OPTPT_OK;
}

int optpt_update_vertices(optpt_renderer *r, const float *positions, const float *normals, void *stream)
{
    if (!r || !positions)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_OR_RETURN(cudaMemcpyAsync(r->dPositions, positions, sizeof(float) * 3 * r->numVerts,
                                   cudaMemcpyHostToDevice, st),
                   "vertex upload");
    if (normals && r->hasNormals)
        CUDA_OR_RETURN(cudaMemcpyAsync(r->dNormals, normals, sizeof(float) * 3 * r->numVerts,
                                       cudaMemcpyHostToDevice, st),
                       "normal upload");
    return afterVertexChange(r, st);
}

int optpt_set_deformation(optpt_renderer *r, const optpt_deformation *d)
{
    if (!r || !d || !d->restPositions || !d->vertexShape)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if (d->numVertices != r->numVerts)
        return fail(OPTPT_ERR_INVALID, "deformation vertex count differs from the scene's");
    if (d->numShapes == 0 || (d->joints && (!d->weights || d->numJoints == 0)))
        return fail(OPTPT_ERR_INVALID, "deformation needs shapes, and weights and joints together");
    for (uint32_t v = 0; v < d->numVertices; ++v) {
        if (d->vertexShape[v] >= d->numShapes)
            return fail(OPTPT_ERR_INVALID, "vertex shape slot out of range");
        if (d->joints)
            for (int k = 0; k < 4; ++k)
                if (d->weights[4 * v + k] != 0.0f && d->joints[4 * v + k] >= d->numJoints)
                    return fail(OPTPT_ERR_INVALID, "joint slot out of range");
    }
    const size_t nv = d->numVertices;
    int rc;
    if ((rc = replaceDevice(r->dRestPos, d->restPositions, 3 * nv, "deformation upload")) ||
        (rc = replaceDevice(r->dRestNrm, r->hasNormals ? d->restNormals : nullptr, 3 * nv, "deformation upload")) ||
        (rc = replaceDevice(r->dVShape, d->vertexShape, nv, "deformation upload")))
        return rc;
    // Joints with zero weight may hold anything; the kernel checks slots, so
    // store zero joints where the weight is zero.
    std::vector<uint16_t> joints;
    if (d->joints) {
        joints.assign(d->joints, d->joints + 4 * nv);
        for (size_t k = 0; k < 4 * nv; ++k)
            if (d->weights[k] == 0.0f)
                joints[k] = 0;
    }
    cudaFree(r->dJoints);
    cudaFree(r->dWeights);
    r->dJoints = r->dWeights = nullptr;
    if (d->joints) {
        CUDA_OR_RETURN(cudaMalloc(&r->dJoints, sizeof(uint16_t) * 4 * nv), "deformation upload");
        CUDA_OR_RETURN(cudaMemcpy(r->dJoints, joints.data(), sizeof(uint16_t) * 4 * nv, cudaMemcpyHostToDevice),
                       "deformation upload");
        CUDA_OR_RETURN(cudaMalloc(&r->dWeights, sizeof(float) * 4 * nv), "deformation upload");
        CUDA_OR_RETURN(cudaMemcpy(r->dWeights, d->weights, sizeof(float) * 4 * nv, cudaMemcpyHostToDevice),
                       "deformation upload");
    }
    cudaFree(r->dShapeM);
    cudaFree(r->dShapeN);
    cudaFree(r->dJointM);
    r->dShapeM = r->dShapeN = r->dJointM = nullptr;
    CUDA_OR_RETURN(cudaMalloc((void **)&r->dShapeM, sizeof(float) * 16 * d->numShapes), "deformation upload");
    CUDA_OR_RETURN(cudaMalloc((void **)&r->dShapeN, sizeof(float) * 9 * d->numShapes), "deformation upload");
    if (d->numJoints)
        CUDA_OR_RETURN(cudaMalloc((void **)&r->dJointM, sizeof(float) * 16 * d->numJoints), "deformation upload");
    r->defVerts = d->numVertices;
    r->defShapes = d->numShapes;
    r->defJoints = d->joints ? d->numJoints : 0;
    return OPTPT_OK;
}

int optpt_deform(optpt_renderer *r, const float *shapeMatrices, const float *shapeNormalMatrices,
                 const float *jointMatrices, void *stream)
{
    if (!r || !shapeMatrices || !shapeNormalMatrices)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if (!r->defVerts)
        return fail(OPTPT_ERR_STATE, "no deformation set (call optpt_set_deformation)");
    if (r->defJoints && !jointMatrices)
        return fail(OPTPT_ERR_INVALID, "joint matrices required for a skinned deformation");
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_OR_RETURN(cudaMemcpyAsync(r->dShapeM, shapeMatrices, sizeof(float) * 16 * r->defShapes,
                                   cudaMemcpyHostToDevice, st),
                   "pose upload");
    CUDA_OR_RETURN(cudaMemcpyAsync(r->dShapeN, shapeNormalMatrices, sizeof(float) * 9 * r->defShapes,
                                   cudaMemcpyHostToDevice, st),
                   "pose upload");
    if (r->defJoints)
        CUDA_OR_RETURN(cudaMemcpyAsync(r->dJointM, jointMatrices, sizeof(float) * 16 * r->defJoints,
                                       cudaMemcpyHostToDevice, st),
                       "pose upload");
    launchDeform(r->defVerts, r->dRestPos, r->dRestNrm, r->dVShape, r->dJoints, r->dWeights, r->dShapeM, r->dShapeN,
                 r->dJointM, r->defShapes, r->defJoints, r->dPositions, r->hasNormals ? r->dNormals : nullptr, st);
    CUDA_OR_RETURN(cudaGetLastError(), "deform kernel");
    return afterVertexChange(r, st);
}

int optpt_refit_profiled(optpt_renderer *r, uint32_t reps, float *msPerRefit)
{
    if (!r || !msPerRefit || reps == 0)
        return fail(OPTPT_ERR_INVALID, "NULL argument or zero repetitions");
    if (!r->bvh.nodes8)
        return fail(OPTPT_ERR_STATE, "refit timing needs the 8-wide BVH");
    cudaStream_t st = r->ownStream;
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "refit profile");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_OR_RETURN(cudaEventCreate(&e0), "refit profile");
    CUDA_OR_RETURN(cudaEventCreate(&e1), "refit profile");
    int err = refitBvh8(r->bvh, r->dPositions, r->dTriIndices, r->scene.numTris, st);  // warm (allocates boxes)
    cudaEventRecord(e0, st);
    for (uint32_t k = 0; k < reps && !err; ++k)
        err = refitBvh8(r->bvh, r->dPositions, r->dTriIndices, r->scene.numTris, st);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err)
        return cudaFail((cudaError_t)err, "refit profile");
    CUDA_OR_RETURN(e, "refit profile");
    *msPerRefit = ms / (float)reps;
    return OPTPT_OK;
}

int optpt_read_vertices(optpt_renderer *r, float *positions, float *normals, void *stream)
{
    if (!r)
        return fail(OPTPT_ERR_INVALID, "NULL renderer");
    cudaStream_t st = (cudaStream_t)stream;
    if (positions)
        CUDA_OR_RETURN(cudaMemcpyAsync(positions, r->dPositions, sizeof(float) * 3 * r->numVerts,
                                       cudaMemcpyDeviceToHost, st),
                       "vertex read");
    if (normals && r->hasNormals)
        CUDA_OR_RETURN(cudaMemcpyAsync(normals, r->dNormals, sizeof(float) * 3 * r->numVerts,
                                       cudaMemcpyDeviceToHost, st),
                       "vertex read");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "vertex read");
    return OPTPT_OK;
}

int optpt_image_out(optpt_renderer *r, uint32_t *rgba8, uint32_t *rgbe, void *halfRows, void *stream)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    launchImageOut(r->acc.frameBuffer, r->acc.accumFrameBuffer, r->w, r->h, rgba8, rgbe, halfRows,
                   (cudaStream_t)stream);
    CUDA_OR_RETURN(cudaGetLastError(), "image output kernel");
    return OPTPT_OK;
}

namespace {

int outScratch(optpt_renderer *r, size_t bytes, void **p)
{
    if (r->outScratchBytes < bytes) {
        cudaFree(r->outScratch);
        r->outScratch = nullptr;
        r->outScratchBytes = 0;
        CUDA_OR_RETURN(cudaMalloc(&r->outScratch, bytes), "image output scratch");
        r->outScratchBytes = bytes;
    }
    *p = r->outScratch;
    return OPTPT_OK;
}

}  // namespace

int optpt_image_out_profiled(optpt_renderer *r, uint32_t reps, float *msPerLaunch)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (!msPerLaunch || reps == 0)
        return fail(OPTPT_ERR_INVALID, "NULL output or zero repetitions");
    const size_t npix = (size_t)r->w * r->h, flushBytes = (size_t)256 << 20;
    void *d = nullptr, *flush = nullptr;
    if ((rc = outScratch(r, npix * 16, &d)))
        return rc;
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "image output profile");
    CUDA_OR_RETURN(cudaMalloc(&flush, flushBytes), "L2 flush buffer");
    cudaStream_t st = r->ownStream;
    uint32_t *rgba8 = (uint32_t *)d, *rgbe = rgba8 + npix;
    void *rows = rgbe + npix;
    std::vector<cudaEvent_t> ev(2 * reps, nullptr);
    cudaError_t e = cudaSuccess;
    for (auto &x : ev)
        if (e == cudaSuccess)
            e = cudaEventCreate(&x);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        launchImageOut(r->acc.frameBuffer, r->acc.accumFrameBuffer, r->w, r->h, rgba8, rgbe, rows, st);
    // Each launch follows a 256 MB write (L2 is 129 MB): it starts cold.
    for (uint32_t k = 0; k < reps && e == cudaSuccess; ++k) {
        cudaMemsetAsync(flush, (int)(k & 0xFF), flushBytes, st);
        cudaEventRecord(ev[2 * k], st);
        launchImageOut(r->acc.frameBuffer, r->acc.accumFrameBuffer, r->w, r->h, rgba8, rgbe, rows, st);
        cudaEventRecord(ev[2 * k + 1], st);
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    float total = 0.0f;
    for (uint32_t k = 0; k < reps && e == cudaSuccess; ++k) {
        float ms = 0.0f;
        e = cudaEventElapsedTime(&ms, ev[2 * k], ev[2 * k + 1]);
        total += ms;
    }
    for (auto &x : ev)
        if (x)
            cudaEventDestroy(x);
    cudaFree(flush);
    CUDA_OR_RETURN(e, "image output profile");
    *msPerLaunch = total / (float)reps;
    return OPTPT_OK;
}

int optpt_read_rgba8(optpt_renderer *r, uint32_t *rgbaHost, void *stream)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (!rgbaHost)
        return fail(OPTPT_ERR_INVALID, "NULL destination");
    void *d = nullptr;
    const size_t bytes = sizeof(uint32_t) * r->w * r->h;
    if ((rc = outScratch(r, bytes, &d)))
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    launchImageOut(r->acc.frameBuffer, nullptr, r->w, r->h, (uint32_t *)d, nullptr, nullptr, st);
    CUDA_OR_RETURN(cudaGetLastError(), "image output kernel");
    CUDA_OR_RETURN(cudaMemcpyAsync(rgbaHost, d, bytes, cudaMemcpyDeviceToHost, st), "rgba8 copy");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "rgba8 copy");
    return OPTPT_OK;
}

int optpt_save_image(optpt_renderer *r, int format, const char *path)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (format < 0 || format > 2)
        return fail(OPTPT_ERR_INVALID, "format must be 0 (PNG), 1 (HDR) or 2 (EXR)");
    static const char *names[3] = {"output.png", "output.hdr", "output.exr"};
    const size_t npix = (size_t)r->w * r->h;
    const size_t bytes = format == 2 ? npix * 8 : npix * 4;
    // The frame may have been rendered on any stream: wait for all of it
    // (the reference's launch() is synchronous, src/renderer.cpp:949).
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "save image");
    void *d = nullptr;
    if ((rc = outScratch(r, bytes, &d)))
        return rc;
    cudaStream_t st = r->ownStream;
    launchImageOut(r->acc.frameBuffer, r->acc.accumFrameBuffer, r->w, r->h, format == 0 ? (uint32_t *)d : nullptr,
                   format == 1 ? (uint32_t *)d : nullptr, format == 2 ? d : nullptr, st);
    CUDA_OR_RETURN(cudaGetLastError(), "image output kernel");
    std::vector<uint8_t> payload(bytes), file;
    CUDA_OR_RETURN(cudaMemcpyAsync(payload.data(), d, bytes, cudaMemcpyDeviceToHost, st), "image payload copy");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "image payload copy");
    const int threads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (format == 0)
        optimg::encodePng(payload.data(), r->w, r->h, (size_t)r->w * 4, file, threads);
    else if (format == 1)
        optimg::encodeHdr(payload.data(), r->w, r->h, file);
    else
        optimg::encodeExr((const uint16_t *)payload.data(), r->w, r->h, 3, file, threads);
    const char *name = path ? path : names[format];
    FILE *f = fopen(name, "wb");
    if (!f)
        return fail(OPTPT_ERR_IO, (std::string("cannot open ") + name + " for writing").c_str());
    const size_t wrote = fwrite(file.data(), 1, file.size(), f);
    const bool ok = fclose(f) == 0 && wrote == file.size();
    if (!ok)
        return fail(OPTPT_ERR_IO, (std::string("cannot write ") + name).c_str());
    return OPTPT_OK;
}

int optpt_read_accum(optpt_renderer *r, double *sumHost, double *sumSqHost, void *stream)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = sizeof(Acc4) * r->w * r->h;
    if (sumHost)
        CUDA_OR_RETURN(cudaMemcpyAsync(sumHost, r->acc.sum, bytes, cudaMemcpyDeviceToHost, st), "accum copy");
    if (sumSqHost)
        CUDA_OR_RETURN(cudaMemcpyAsync(sumSqHost, r->acc.sumSq, bytes, cudaMemcpyDeviceToHost, st), "accum copy");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "accum copy");
    return OPTPT_OK;
}

int optpt_get_stats(optpt_renderer *r, optpt_stats *out)
{
    if (!r || !out)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    unsigned long long t[TOTALS_COUNT] = {};
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "stats");
    CUDA_OR_RETURN(cudaMemcpy(t, r->q.totals, sizeof(t), cudaMemcpyDeviceToHost), "stats");
    out->extensionRays = t[0];
    out->shadowRays = t[1];
    out->pathSamples = t[2];
    out->nanSamples = t[3];
    out->traversalStackOverflows = t[8];
    out->traversalBudgetExhausted = t[9];
    out->bvh8Levels = (uint32_t)r->bvh.levels8;
    out->tailBounce = r->tailBounce <= r->lp.maxDepth ? r->tailBounce : 0u;
    out->bvhNodes = (uint32_t)r->bvh.usedNodes;
    out->bvhLeaves = (uint32_t)r->bvh.numLeaves;
    out->bvh8Nodes = (uint32_t)r->bvh.numNodes8;
    out->bvhWidth = r->bvh.nodes8 ? 8u : 2u;
    out->sppBatch = r->sppBatch;
    out->blockSize = (uint32_t)r->shape.block;
    return OPTPT_OK;
}

int optpt_render_profiled(optpt_renderer *r, uint32_t spp, void *stream, optpt_kernel_times *out)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (!out)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    memset(out, 0, sizeof(*out));
    if ((rc = ensureGuideBuffers(r)))
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const FrameParams fp = r->frameParams();
    const int maxEv = 4 + 4 * (int)fp.maxDepth;
    std::vector<cudaEvent_t> ev(maxEv);
    std::vector<int> kind(maxEv);
    for (auto &e : ev)
        CUDA_OR_RETURN(cudaEventCreate(&e), "event");
    unsigned long long before[2] = {0, 0}, after[2] = {0, 0};
    CUDA_OR_RETURN(r->uploadFrameConst(st), "frame constants");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "profile");
    CUDA_OR_RETURN(cudaMemcpy(before, r->q.totals, sizeof(before), cudaMemcpyDeviceToHost), "profile");
    const uint32_t passes = (spp + r->sppBatch - 1) / r->sppBatch;
    for (uint32_t p = 0; p < passes; ++p) {
        FrameParams pf = fp;
        if (p + 1 == passes && spp % r->sppBatch) {
            pf.sppBatch = spp % r->sppBatch;
            pf.numPaths = r->w * r->h * pf.sppBatch;
        }
        const int marks = enqueuePass(r, pf, st, ev.data(), kind.data());
        CUDA_OR_RETURN(cudaStreamSynchronize(st), "profile pass");
        for (int k = 0; k + 1 < marks; ++k) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            out->ms[kind[k]] += ms;
            out->launches[kind[k]] += kind[k] == 3 ? 2 : kind[k] == 6 ? 1 + 5 * r->gTrainSteps : 1;
        }
    }
    r->lp.sample += spp;
    r->hostFbValid = false;
    CUDA_OR_RETURN(cudaMemcpy(after, r->q.totals, sizeof(after), cudaMemcpyDeviceToHost), "profile");
    out->extensionRays = after[0] - before[0];
    out->shadowRays = after[1] - before[1];
    for (auto &e : ev)
        cudaEventDestroy(e);
    return OPTPT_OK;
}

int optpt_traversal_counts(optpt_renderer *r, uint32_t spp, void *stream, optpt_traversal_work *out)
{
    int rc = checkRenderable(r);
    if (rc)
        return rc;
    if (!out)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if ((rc = ensureGuideBuffers(r)))
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long before[8], after[8];
    CUDA_OR_RETURN(r->uploadFrameConst(st), "frame constants");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "counts");
    CUDA_OR_RETURN(cudaMemcpy(before, r->q.totals, sizeof(before), cudaMemcpyDeviceToHost), "counts");
    const FrameParams fp = r->frameParams();
    for (uint32_t done = 0; done < spp;) {
        FrameParams pf = fp;
        pf.sppBatch = spp - done < r->sppBatch ? spp - done : r->sppBatch;
        pf.numPaths = r->w * r->h * pf.sppBatch;
        enqueuePass(r, pf, st, nullptr, nullptr, true);
        done += pf.sppBatch;
    }
    CUDA_OR_RETURN(cudaGetLastError(), "counts launch");
    CUDA_OR_RETURN(cudaStreamSynchronize(st), "counts");
    CUDA_OR_RETURN(cudaMemcpy(after, r->q.totals, sizeof(after), cudaMemcpyDeviceToHost), "counts");
    r->lp.sample += spp;
    r->hostFbValid = false;
    out->extensionRays = after[0] - before[0];
    out->shadowRays = after[1] - before[1];
    out->extensionNodes = after[4] - before[4];
    out->extensionTris = after[5] - before[5];
    out->shadowNodes = after[6] - before[6];
    out->shadowTris = after[7] - before[7];
    return OPTPT_OK;
}

int optpt_trace(optpt_renderer *r, const float *rays, float *hits, uint32_t n, int anyHit, void *stream)
{
    if (!r || (n && (!rays || !hits)))
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    if (r->numTris == 0) {
        std::vector<float4> miss(n, make_float4(INFINITY, 0.0f, 0.0f, 0.0f));
        for (auto &m : miss) {
            int neg = -1;
            memcpy(&m.w, &neg, 4);
        }
        CUDA_OR_RETURN(cudaMemcpyAsync(hits, miss.data(), sizeof(float4) * n, cudaMemcpyHostToDevice,
                                       (cudaStream_t)stream),
                       "trace");
        CUDA_OR_RETURN(cudaStreamSynchronize((cudaStream_t)stream), "trace");
        return OPTPT_OK;
    }
    launchTrace(r->scene, (const float4 *)rays, (float4 *)hits, n, anyHit, r->q.totals, (cudaStream_t)stream);
    CUDA_OR_RETURN(cudaGetLastError(), "trace launch");
    return OPTPT_OK;
}

int optpt_bvh_leaf_order(optpt_renderer *r, uint32_t *mortonSorted, int32_t *primOrder)
{
    if (!r)
        return fail(OPTPT_ERR_INVALID, "renderer is NULL");
    if (r->numTris == 0)
        return OPTPT_OK;
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "leaf order");
    if (mortonSorted)
        CUDA_OR_RETURN(cudaMemcpy(mortonSorted, r->bvh.mortonSorted, sizeof(uint32_t) * r->numTris,
                                  cudaMemcpyDeviceToHost),
                       "leaf order");
    if (primOrder)
        CUDA_OR_RETURN(cudaMemcpy(primOrder, r->bvh.primOrder, sizeof(int32_t) * r->numTris, cudaMemcpyDeviceToHost),
                       "leaf order");
    return OPTPT_OK;
}

int optpt_bvh8_nodes(optpt_renderer *r, void *nodes, uint32_t capacity, uint32_t *numNodes, int32_t *primOrder8)
{
    if (!r || !numNodes)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    *numNodes = (uint32_t)r->bvh.numNodes8;
    if (r->bvh.nodes8 == nullptr)
        return OPTPT_OK;
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "bvh8");
    if (nodes) {
        if (capacity < (uint32_t)r->bvh.numNodes8)
            return fail(OPTPT_ERR_INVALID, "capacity below the node count");
        CUDA_OR_RETURN(cudaMemcpy(nodes, r->bvh.nodes8, 80ull * r->bvh.numNodes8, cudaMemcpyDeviceToHost), "bvh8");
    }
    if (primOrder8) {
        std::vector<float4> tv(3 * (size_t)r->numTris);
        CUDA_OR_RETURN(cudaMemcpy(tv.data(), r->bvh.triV8, sizeof(float4) * tv.size(), cudaMemcpyDeviceToHost), "bvh8");
        for (int i = 0; i < r->numTris; ++i)
            memcpy(&primOrder8[i], &tv[3 * i].w, 4);
    }
    return OPTPT_OK;
}

int optpt_bvh_nodes(optpt_renderer *r, int32_t *nodes4, uint32_t capacity, uint32_t *numNodes)
{
    if (!r || !numNodes)
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    *numNodes = (uint32_t)r->bvh.numNodes;
    if (!nodes4 || r->bvh.numNodes == 0)
        return OPTPT_OK;
    if (capacity < (uint32_t)r->bvh.numNodes)
        return fail(OPTPT_ERR_INVALID, "capacity below the node count");
    std::vector<BvhNode> nodes(r->bvh.numNodes);
    CUDA_OR_RETURN(cudaDeviceSynchronize(), "nodes");
    CUDA_OR_RETURN(cudaMemcpy(nodes.data(), r->bvh.nodes, sizeof(BvhNode) * nodes.size(), cudaMemcpyDeviceToHost),
                   "nodes");
    for (size_t i = 0; i < nodes.size(); ++i) {
        nodes4[4 * i] = nodes[i].d.x;
        nodes4[4 * i + 1] = nodes[i].d.y;
        nodes4[4 * i + 2] = nodes[i].d.z;
        nodes4[4 * i + 3] = nodes[i].d.w;
    }
    return OPTPT_OK;
}

int optpt_bsdf_batch(const optpt_bsdf_query *queries, optpt_bsdf_result *results, uint32_t n, void *stream)
{
    if (n && (!queries || !results))
        return fail(OPTPT_ERR_INVALID, "NULL argument");
    launchBsdfBatch(queries, results, n, (cudaStream_t)stream);
    CUDA_OR_RETURN(cudaGetLastError(), "bsdf launch");
    return OPTPT_OK;
}

}  // extern "C"
