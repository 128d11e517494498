// frame.cu — the whole per-frame pipeline of the reference application (app/src/main.cpp:
// 126-160: track against the previous raycast, integrate at the tracked pose, raycast at that
// pose) as one CUDA graph with the pose kept on the device.
//
// The graph is captured once per mode (with / without tracking) on a private stream and then
// launched on the caller's stream: 31 kernels for a tracked frame with no host round trip.
// ICP iterations after convergence return at entry, so the fixed launch sequence reproduces
// the reference's early exit. The frame counter (the integration timestamp) lives on the
// device and advances by one per launch.
#include <cstring>

#include "pipeline.cuh"
#include "profile.cuh"
#include "se_gpu_internal.cuh"

namespace se_gpu {
int tracker_accepted_offset();
void* tracker_state(se_gpu_tracker* t);

// The autotuner's candidates: update grid 4, 8 or 16 CTAs per SM with 4 or 2 voxels per lane
// per round (update candidate u), raycast warp tile 8 x 4 or 16 x 2 (raycast candidate r).
constexpr int kUpdateCandidates = 6, kRaycastCandidates = 2;
static FrameTiles tune_candidate(int u, int r)
{
    static const int ctas[3] = {4, 8, 16};
    FrameTiles t;
    t.update_ctas_per_sm = ctas[u % 3];
    t.update_round = u < 3 ? 4 : 2;
    t.raycast_tile = r;
    return t;
}

// The acceptance of a run that did not track: copied on the stream like a tracked run's flag,
// so that it lands in stream order after any earlier read into the same host buffer.
static __device__ int g_accepted_untracked = 1; // never written
} // namespace se_gpu

using namespace se_gpu;

struct se_gpu_frame {
    se_gpu_map* map;
    se_gpu_tracker* tracker; // may be null: integrate + raycast only
    se_gpu_pinhole sensor;
    float* pose12;           // device T_WS (row-major 3x4)
    float* depth;            // device input depth, width * height
    float* depth_filtered;   // the bilateral-filtered tracking input (when enabled)
    int bilateral;
    se_gpu_bilateral_config bilateral_config;
    float* pts;              // device raycast points (the next frame's tracking reference)
    float* nrm;
    int8_t* scale;
    cudaStream_t capture_stream;
    cudaGraphExec_t exec[2]; // [0] integrate + raycast, [1] track + integrate + raycast
    int last_tracked;        // whether the last run tracked (acceptance is 1 otherwise)
    // autotuner: the runs left to time, the events, and per candidate the least time seen
    int tune_left, tune_done;
    FrameTuneEvents* tune_ev;
    float update_ms[kUpdateCandidates];
    float raycast_ms[kRaycastCandidates];
    // host inputs: two device staging slots filled on a copy stream, so that the next frame's
    // copy runs while this frame computes; the frame's stream copies a slot into `depth`
    float* staging[2];
    cudaStream_t copy_stream;
    cudaEvent_t copied[2], consumed[2];
    int slot;
};

// One frame's launches on stream (captured into the graph, or run directly while tuning).
static se_gpu_status enqueue_frame(se_gpu_frame* f, int with_track, cudaStream_t stream)
{
    se_gpu_status st = SE_GPU_OK;
    const float* track_in = f->depth;
    if (with_track && f->bilateral) {
        st = enqueue_bilateral(f->depth, f->depth_filtered, f->sensor.width, f->sensor.height, f->bilateral_config,
                               stream);
        track_in = f->depth_filtered;
    }
    if (with_track && st == SE_GPU_OK)
        st = enqueue_track(f->tracker, track_in, f->pts, f->nrm, nullptr, f->pose12, stream);
    if (st == SE_GPU_OK)
        st = enqueue_integrate(f->map, f->depth, f->sensor, nullptr, f->pose12, 0, stream);
    if (st == SE_GPU_OK)
        st = enqueue_raycast(f->map, f->sensor, nullptr, f->pose12, f->pts, f->nrm, f->scale, stream);
    return st;
}

static se_gpu_status capture(se_gpu_frame* f, int with_track)
{
    cudaGraph_t graph = nullptr;
    profiling_suspend(true);
    cudaError_t e = cudaStreamBeginCapture(f->capture_stream, cudaStreamCaptureModeThreadLocal);
    se_gpu_status st = SE_GPU_OK;
    if (e == cudaSuccess) {
        st = enqueue_frame(f, with_track, f->capture_stream);
        const cudaError_t e2 = cudaStreamEndCapture(f->capture_stream, &graph);
        if (e2 != cudaSuccess && st == SE_GPU_OK)
            st = cuda_status(e2, "cudaStreamEndCapture");
    }
    else {
        st = cuda_status(e, "cudaStreamBeginCapture");
    }
    profiling_suspend(false);
    if (st != SE_GPU_OK) {
        if (graph)
            cudaGraphDestroy(graph);
        return st;
    }
    e = cudaGraphInstantiate(&f->exec[with_track], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_status(e, "cudaGraphInstantiate");
    return SE_GPU_OK;
}

extern "C" {

se_gpu_status se_gpu_frame_create(se_gpu_map* map, se_gpu_tracker* tracker, const se_gpu_pinhole* sensor,
                                  se_gpu_frame** out)
{
    if (!map || !sensor || !out || sensor->width <= 0 || sensor->height <= 0) {
        set_last_error("se_gpu_frame_create: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (map->occ) {
        set_last_error("se_gpu_frame_create: TSDF maps only");
        return SE_GPU_ERR_NOT_SUPPORTED;
    }
    se_gpu_frame* f = new se_gpu_frame();
    std::memset(f, 0, sizeof(*f));
    f->map = map;
    f->tracker = tracker;
    f->sensor = *sensor;
    const size_t npx = (size_t) sensor->width * sensor->height;
    auto fail = [&](cudaError_t e, const char* what) {
        se_gpu_status st = cuda_status(e, what);
        se_gpu_frame_destroy(f);
        return st;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&f->pose12, 12 * sizeof(float))) != cudaSuccess) return fail(e, "cudaMalloc(pose)");
    if ((e = cudaMalloc(&f->depth, npx * sizeof(float))) != cudaSuccess) return fail(e, "cudaMalloc(depth)");
    if ((e = cudaMalloc(&f->pts, npx * 3 * sizeof(float))) != cudaSuccess) return fail(e, "cudaMalloc(points)");
    if ((e = cudaMalloc(&f->nrm, npx * 3 * sizeof(float))) != cudaSuccess) return fail(e, "cudaMalloc(normals)");
    if ((e = cudaMalloc(&f->scale, npx)) != cudaSuccess) return fail(e, "cudaMalloc(scale)");
    if ((e = cudaMemset(f->pts, 0, npx * 3 * sizeof(float))) != cudaSuccess) return fail(e, "cudaMemset");
    if ((e = cudaMemset(f->nrm, 0, npx * 3 * sizeof(float))) != cudaSuccess) return fail(e, "cudaMemset");
    if ((e = cudaStreamCreateWithFlags(&f->capture_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(e, "cudaStreamCreate");
    if ((e = cudaStreamCreateWithFlags(&f->copy_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return fail(e, "cudaStreamCreate");
    for (int i = 0; i < 2; ++i) {
        if ((e = cudaMalloc(&f->staging[i], npx * sizeof(float))) != cudaSuccess) return fail(e, "cudaMalloc(staging)");
        if ((e = cudaEventCreateWithFlags(&f->copied[i], cudaEventDisableTiming)) != cudaSuccess)
            return fail(e, "cudaEventCreate");
        if ((e = cudaEventCreateWithFlags(&f->consumed[i], cudaEventDisableTiming)) != cudaSuccess)
            return fail(e, "cudaEventCreate");
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e, "cudaDeviceSynchronize");
    *out = f;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_destroy(se_gpu_frame* f)
{
    if (!f)
        return SE_GPU_OK;
    for (int i = 0; i < 2; ++i)
        if (f->exec[i])
            cudaGraphExecDestroy(f->exec[i]);
    if (f->capture_stream)
        cudaStreamDestroy(f->capture_stream);
    if (f->copy_stream)
        cudaStreamDestroy(f->copy_stream);
    for (int i = 0; i < 2; ++i) {
        cudaFree(f->staging[i]);
        if (f->copied[i])
            cudaEventDestroy(f->copied[i]);
        if (f->consumed[i])
            cudaEventDestroy(f->consumed[i]);
    }
    if (f->tune_ev) {
        for (int i = 0; i < 4; ++i)
            if (f->tune_ev->ev[i])
                cudaEventDestroy(f->tune_ev->ev[i]);
        delete f->tune_ev;
    }
    cudaFree(f->pose12);
    cudaFree(f->depth);
    cudaFree(f->depth_filtered);
    cudaFree(f->pts);
    cudaFree(f->nrm);
    cudaFree(f->scale);
    delete f;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_buffers(se_gpu_frame* f, float** depth_dev, float** pts_W_dev, float** nrm_W_dev,
                                   int8_t** scale_dev)
{
    if (!f) {
        set_last_error("se_gpu_frame_buffers: null frame");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (depth_dev)
        *depth_dev = f->depth;
    if (pts_W_dev)
        *pts_W_dev = f->pts;
    if (nrm_W_dev)
        *nrm_W_dev = f->nrm;
    if (scale_dev)
        *scale_dev = f->scale;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_set_pose(se_gpu_frame* f, const float T_WS[16], int timestamp)
{
    if (!f || !T_WS) {
        set_last_error("se_gpu_frame_set_pose: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    SE_CUDA_TRY(cudaDeviceSynchronize());
    SE_CUDA_TRY(cudaMemcpy(f->pose12, T_WS, 12 * sizeof(float), cudaMemcpyHostToDevice));
    SE_CUDA_TRY(cudaMemcpy(f->map->timestamp_dev, &timestamp, sizeof(int), cudaMemcpyHostToDevice));
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_set_bilateral(se_gpu_frame* f, const se_gpu_bilateral_config* config)
{
    if (!f) {
        set_last_error("se_gpu_frame_set_bilateral: null frame");
        return SE_GPU_ERR_BAD_ARG;
    }
    if (config) {
        const se_gpu_status st = check_bilateral(config);
        if (st != SE_GPU_OK)
            return st;
        if (!f->depth_filtered)
            SE_CUDA_TRY(cudaMalloc(&f->depth_filtered, (size_t) f->sensor.width * f->sensor.height * sizeof(float)));
        f->bilateral_config = *config;
    }
    f->bilateral = config ? 1 : 0;
    // the tracked graph changes; a frame in flight keeps its own executable until it completes
    if (f->exec[1]) {
        SE_CUDA_TRY(cudaDeviceSynchronize());
        cudaGraphExecDestroy(f->exec[1]);
        f->exec[1] = nullptr;
    }
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_run(se_gpu_frame* f, int track, void* stream_p)
{
    if (!f || (track && !f->tracker)) {
        set_last_error("se_gpu_frame_run: invalid argument (tracking needs a tracker)");
        return SE_GPU_ERR_BAD_ARG;
    }
    const int mode = track ? 1 : 0;
    cudaStream_t stream = (cudaStream_t) stream_p;
    if (f->tune_left > 0) {
        // a tuning run: the launches directly on the stream with the next candidate geometry,
        // the update and raycast timed with events (the run synchronises the stream)
        const int k = f->tune_done++;
        const int u = k % kUpdateCandidates, r = k % kRaycastCandidates;
        f->map->tiles = tune_candidate(u, r);
        f->map->tune = f->tune_ev;
        f->map->last_stream = stream;
        f->last_tracked = mode;
        const se_gpu_status st = enqueue_frame(f, mode, stream);
        f->map->tune = nullptr;
        if (st != SE_GPU_OK)
            return st;
        SE_CUDA_TRY(cudaEventSynchronize(f->tune_ev->ev[3]));
        float up = 0.0f, rc = 0.0f;
        SE_CUDA_TRY(cudaEventElapsedTime(&up, f->tune_ev->ev[0], f->tune_ev->ev[1]));
        SE_CUDA_TRY(cudaEventElapsedTime(&rc, f->tune_ev->ev[2], f->tune_ev->ev[3]));
        f->update_ms[u] = up < f->update_ms[u] ? up : f->update_ms[u];
        f->raycast_ms[r] = rc < f->raycast_ms[r] ? rc : f->raycast_ms[r];
        if (--f->tune_left == 0) {
            int bu = 0, br = 0;
            for (int c = 1; c < kUpdateCandidates; ++c)
                bu = f->update_ms[c] < f->update_ms[bu] ? c : bu;
            for (int c = 1; c < kRaycastCandidates; ++c)
                br = f->raycast_ms[c] < f->raycast_ms[br] ? c : br;
            f->map->tiles = tune_candidate(bu, br);
            // the graphs are captured again with the chosen geometry
            for (int i = 0; i < 2; ++i)
                if (f->exec[i]) {
                    SE_CUDA_TRY(cudaGraphExecDestroy(f->exec[i]));
                    f->exec[i] = nullptr;
                }
        }
        return SE_GPU_OK;
    }
    if (!f->exec[mode]) {
        const se_gpu_status st = capture(f, mode);
        if (st != SE_GPU_OK)
            return st;
    }
    f->map->last_stream = stream;
    f->last_tracked = mode;
    ProfScope ps(kProfFrameGraph, stream);
    SE_CUDA_TRY(cudaGraphLaunch(f->exec[mode], stream));
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_autotune(se_gpu_frame* f, int runs)
{
    if (!f || runs < 0 || runs > 1000 || (runs > 0 && runs < kUpdateCandidates)) {
        set_last_error("se_gpu_frame_autotune: invalid argument (0 or %d..1000 runs)", kUpdateCandidates);
        return SE_GPU_ERR_BAD_ARG;
    }
    if (runs > 0 && !f->tune_ev) {
        f->tune_ev = new FrameTuneEvents();
        for (int i = 0; i < 4; ++i)
            SE_CUDA_TRY(cudaEventCreate(&f->tune_ev->ev[i]));
    }
    for (int c = 0; c < kUpdateCandidates; ++c)
        f->update_ms[c] = 1e30f;
    for (int c = 0; c < kRaycastCandidates; ++c)
        f->raycast_ms[c] = 1e30f;
    f->tune_left = runs;
    f->tune_done = 0;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_tiles(const se_gpu_frame* f, int tiles[3], int* tuning_left)
{
    if (!f || !tiles) {
        set_last_error("se_gpu_frame_tiles: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    tiles[0] = f->map->tiles.update_ctas_per_sm;
    tiles[1] = f->map->tiles.update_round;
    tiles[2] = f->map->tiles.raycast_tile;
    if (tuning_left)
        *tuning_left = f->tune_left;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_run_host(se_gpu_frame* f, const float* depth_host, int track, void* stream_p)
{
    if (!f || !depth_host) {
        set_last_error("se_gpu_frame_run_host: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    const size_t bytes = (size_t) f->sensor.width * (size_t) f->sensor.height * sizeof(float);
    cudaStream_t stream = (cudaStream_t) stream_p;
    // the host copy on the copy stream into a staging slot (free once the frame stream's copy out
    // of it from two calls ago has run), then the device copy on the frame's stream
    const int k = f->slot;
    f->slot ^= 1;
    SE_CUDA_TRY(cudaStreamWaitEvent(f->copy_stream, f->consumed[k], 0));
    SE_CUDA_TRY(cudaMemcpyAsync(f->staging[k], depth_host, bytes, cudaMemcpyHostToDevice, f->copy_stream));
    SE_CUDA_TRY(cudaEventRecord(f->copied[k], f->copy_stream));
    SE_CUDA_TRY(cudaStreamWaitEvent(stream, f->copied[k], 0));
    SE_CUDA_TRY(cudaMemcpyAsync(f->depth, f->staging[k], bytes, cudaMemcpyDeviceToDevice, stream));
    SE_CUDA_TRY(cudaEventRecord(f->consumed[k], stream));
    return se_gpu_frame_run(f, track, stream_p);
}

se_gpu_status se_gpu_frame_get_pose(se_gpu_frame* f, float T_WS[16], int* accepted, void* stream_p)
{
    if (!f || !T_WS) {
        set_last_error("se_gpu_frame_get_pose: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    SE_CUDA_TRY(cudaMemcpyAsync(T_WS, f->pose12, 12 * sizeof(float), cudaMemcpyDeviceToHost, stream));
    int acc = 1;
    if (accepted && f->tracker && f->last_tracked)
        SE_CUDA_TRY(cudaMemcpyAsync(&acc, (char*) tracker_state(f->tracker) + tracker_accepted_offset(), sizeof(int),
                                    cudaMemcpyDeviceToHost, stream));
    SE_CUDA_TRY(cudaStreamSynchronize(stream));
    T_WS[12] = T_WS[13] = T_WS[14] = 0.0f;
    T_WS[15] = 1.0f;
    if (accepted)
        *accepted = acc;
    return SE_GPU_OK;
}

se_gpu_status se_gpu_frame_get_pose_async(se_gpu_frame* f, float pose12_host[12], int* accepted_host, void* stream_p)
{
    if (!f || !pose12_host || !accepted_host) {
        set_last_error("se_gpu_frame_get_pose_async: invalid argument");
        return SE_GPU_ERR_BAD_ARG;
    }
    cudaStream_t stream = (cudaStream_t) stream_p;
    SE_CUDA_TRY(cudaMemcpyAsync(pose12_host, f->pose12, 12 * sizeof(float), cudaMemcpyDeviceToHost, stream));
    if (f->tracker && f->last_tracked)
        SE_CUDA_TRY(cudaMemcpyAsync(accepted_host, (char*) tracker_state(f->tracker) + tracker_accepted_offset(),
                                    sizeof(int), cudaMemcpyDeviceToHost, stream));
    else
        SE_CUDA_TRY(cudaMemcpyFromSymbolAsync(accepted_host, g_accepted_untracked, sizeof(int), 0,
                                              cudaMemcpyDeviceToHost, stream));
    return SE_GPU_OK;
}

} // extern "C"
