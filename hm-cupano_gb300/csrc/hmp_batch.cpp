// hmp_batch.cpp -- a batched job: many process() calls of several stitchers, captured once into a
// CUDA graph and replayed with one launch (hmp_batch_*, include/hmpano.h).
//
// Calls added under the same stream index run in the order they were added; different stream
// indices run concurrently (one internal stream each, forked from and joined to the launch
// stream). The first capture runs the job once eagerly, so that first-call work (the canvas
// planes resolved for the frames' geometry) happens outside the graph; the graph then holds only
// the per-frame kernels. Inputs and canvases are device pointers fixed at add time: a replay
// reads and writes the same buffers, so callers refill the inputs between launches.
#include <cuda_runtime.h>

#include <cstdio>
#include <new>
#include <string>
#include <vector>

#include "hmpano.h"

namespace {

hmp_status bstatus(int code, const std::string& msg) {
  hmp_status s;
  s.code = code;
  std::snprintf(s.message, sizeof(s.message), "%s", msg.c_str());
  return s;
}

hmp_status cstatus(cudaError_t e, const char* what) {
  return bstatus(int(e), std::string(what) + ": " + cudaGetErrorString(e));
}

struct Call {
  hmp_stitcher* st;
  std::vector<hmp_image> inputs;
  hmp_image canvas;
};

}  // namespace

struct hmp_batch {
  std::vector<std::vector<Call>> streams;  // by stream index
  std::vector<cudaStream_t> cs;
  cudaStream_t cap = nullptr;  // the graph is captured on this stream (any launch stream may replay it)
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;

  ~hmp_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    for (cudaStream_t s : cs) cudaStreamDestroy(s);
    if (cap) cudaStreamDestroy(cap);
  }

  hmp_status prepare() {
    while (cs.size() < streams.size()) {
      cudaStream_t s;
      cudaEvent_t e;
      cudaError_t r = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
      if (r != cudaSuccess) return cstatus(r, "batch stream");
      cs.push_back(s);
      r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
      if (r != cudaSuccess) return cstatus(r, "batch event");
      joins.push_back(e);
    }
    if (!fork) {
      const cudaError_t r = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
      if (r != cudaSuccess) return cstatus(r, "batch event");
    }
    if (!cap) {
      const cudaError_t r = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
      if (r != cudaSuccess) return cstatus(r, "batch stream");
    }
    return bstatus(HMP_OK, "");
  }

  // Every call, each stream index on its own stream, forked from and joined back to `root`.
  hmp_status enqueue(cudaStream_t root) {
    cudaError_t r = cudaEventRecord(fork, root);
    if (r != cudaSuccess) return cstatus(r, "batch fork");
    for (size_t i = 0; i < streams.size(); ++i) {
      if (streams[i].empty()) continue;
      r = cudaStreamWaitEvent(cs[i], fork, 0);
      if (r != cudaSuccess) return cstatus(r, "batch fork");
      for (const Call& c : streams[i]) {
        const hmp_status s = hmp_stitcher_process(c.st, c.inputs.data(), int(c.inputs.size()), &c.canvas, cs[i]);
        if (s.code != HMP_OK) return s;
      }
      r = cudaEventRecord(joins[i], cs[i]);
      if (r == cudaSuccess) r = cudaStreamWaitEvent(root, joins[i], 0);
      if (r != cudaSuccess) return cstatus(r, "batch join");
    }
    return bstatus(HMP_OK, "");
  }
};

extern "C" {

HMP_API hmp_status hmp_batch_create(hmp_batch** out) {
  if (!out) return bstatus(HMP_ERR_INVALID_VALUE, "null argument");
  *out = new (std::nothrow) hmp_batch;
  return *out ? bstatus(HMP_OK, "") : bstatus(HMP_ERR_MEMORY_ALLOCATION, "out of host memory");
}

HMP_API void hmp_batch_destroy(hmp_batch* b) { delete b; }

HMP_API hmp_status hmp_batch_add(hmp_batch* b, hmp_stitcher* st, const hmp_image* inputs, int n_inputs,
                                 const hmp_image* canvas, int stream_index) {
  if (!b || !st || !inputs || !canvas || n_inputs < 1 || stream_index < 0 || stream_index > 255)
    return bstatus(HMP_ERR_INVALID_VALUE, "batch add: null argument or stream index outside 0..255");
  if (b->exec) return bstatus(HMP_ERR_INVALID_VALUE, "batch add: the job is already captured");
  // A stitcher holds one frame's intermediate levels: its calls must run in order, on one stream.
  for (size_t i = 0; i < b->streams.size(); ++i)
    for (const Call& c : b->streams[i])
      if (c.st == st && int(i) != stream_index)
        return bstatus(HMP_ERR_INVALID_VALUE, "batch add: a stitcher's calls must share one stream index");
  if (size_t(stream_index) >= b->streams.size()) b->streams.resize(size_t(stream_index) + 1);
  b->streams[size_t(stream_index)].push_back(Call{st, std::vector<hmp_image>(inputs, inputs + n_inputs), *canvas});
  return bstatus(HMP_OK, "");
}

HMP_API hmp_status hmp_batch_capture(hmp_batch* b, void* stream) {
  if (!b) return bstatus(HMP_ERR_INVALID_VALUE, "batch is null");
  if (b->exec) return bstatus(HMP_OK, "");
  const cudaStream_t root = static_cast<cudaStream_t>(stream);
  hmp_status s = b->prepare();
  if (s.code != HMP_OK) return s;
  s = b->enqueue(root);  // eager run: first-call work stays out of the graph
  if (s.code != HMP_OK) return s;
  cudaError_t r = cudaStreamSynchronize(root);
  if (r != cudaSuccess) return cstatus(r, "batch warm-up");
  // Captured on the batch's own stream: the legacy default stream cannot be captured, and the
  // graph does not depend on the stream it was captured on.
  r = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
  if (r != cudaSuccess) return cstatus(r, "batch capture");
  s = b->enqueue(b->cap);
  cudaGraph_t g = nullptr;
  r = cudaStreamEndCapture(b->cap, &g);
  if (s.code != HMP_OK) {
    if (g) cudaGraphDestroy(g);
    return s;
  }
  if (r != cudaSuccess) return cstatus(r, "batch capture");
  b->graph = g;
  r = cudaGraphInstantiate(&b->exec, g, 0);
  if (r != cudaSuccess) {
    b->exec = nullptr;
    return cstatus(r, "batch graph instantiate");
  }
  return bstatus(HMP_OK, "");
}

HMP_API hmp_status hmp_batch_launch(hmp_batch* b, void* stream) {
  if (!b) return bstatus(HMP_ERR_INVALID_VALUE, "batch is null");
  if (!b->exec) {
    const hmp_status s = hmp_batch_capture(b, stream);
    if (s.code != HMP_OK) return s;
  }
  const cudaError_t r = cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream));
  return r == cudaSuccess ? bstatus(HMP_OK, "") : cstatus(r, "batch launch");
}

}  // extern "C"
