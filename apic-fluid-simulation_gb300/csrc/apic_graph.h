// apic_graph.h — building CUDA graphs with device-side loops.
//
// The substep loop of Apic::update (src/apic.rs:2432) and the PCG iteration
// loop (:1899) have data-dependent trip counts.  They become conditional WHILE
// nodes whose condition a small control kernel sets on the device
// (cudaGraphSetConditional), so one update is one graph launch with no host
// round trip.  Kernel sequences are recorded into a graph with
// cudaStreamBeginCaptureToGraph; a cursor keeps the graph's current leaf nodes
// so conditional nodes and further captures chain after them.
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "apic_internal.h"

namespace apic {

struct GraphCursor {
    cudaGraph_t g = nullptr;
    std::vector<cudaGraphNode_t> tail;
};

// Record the launches that `f` enqueues on the capture stream `cap` as nodes
// of c.g after c.tail.
template <class F> cudaError_t capture_on(cudaStream_t cap, GraphCursor& c, F&& f) {
    cudaError_t e = cudaStreamBeginCaptureToGraph(cap, c.g, c.tail.empty() ? nullptr : c.tail.data(), nullptr,
                                                  c.tail.size(), cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return e;
    cudaError_t fe = f();
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t ge = cudaStreamGetCaptureInfo(cap, &st, nullptr, nullptr, &deps, nullptr, &nd);
    std::vector<cudaGraphNode_t> nt;
    if (ge == cudaSuccess && deps) nt.assign(deps, deps + nd);
    cudaGraph_t out = nullptr;
    cudaError_t ee = cudaStreamEndCapture(cap, &out);
    if (fe != cudaSuccess) return fe;
    if (ge != cudaSuccess) return ge;
    if (ee != cudaSuccess) return ee;
    if (!nt.empty()) c.tail = nt;
    return cudaSuccess;
}

// Record the launches that `f` enqueues on s.stream as nodes of c.g after c.tail.
template <class F> cudaError_t capture_into(Scene& s, GraphCursor& c, F&& f) {
    cudaStream_t saved = s.stream;
    s.stream = s.cap_stream;
    cudaError_t e = capture_on(s.cap_stream, c, [&]() { return f(); });
    s.stream = saved;
    return e;
}

// Append a conditional node (IF or WHILE) after c.tail for handle h (created
// on c.g beforehand, so the control kernel that sets it can be captured first);
// `body` receives the node's body graph.
inline cudaError_t add_conditional_with(GraphCursor& c, cudaGraphConditionalNodeType type,
                                        cudaGraphConditionalHandle h, GraphCursor* body) {
    // cudaGraphNodeParams holds a union without a default constructor: zeroed storage
    alignas(cudaGraphNodeParams) unsigned char buf[sizeof(cudaGraphNodeParams)];
    std::memset(buf, 0, sizeof(buf));
    cudaGraphNodeParams* p = reinterpret_cast<cudaGraphNodeParams*>(buf);
    p->type = cudaGraphNodeTypeConditional;
    p->conditional.handle = h;
    p->conditional.type = type;
    p->conditional.size = 1;
    cudaGraphNode_t n;
    cudaError_t e = cudaGraphAddNode(&n, c.g, c.tail.empty() ? nullptr : c.tail.data(), nullptr, c.tail.size(), p);
    if (e != cudaSuccess) return e;
    c.tail.assign(1, n);
    body->g = p->conditional.phGraph_out[0];
    body->tail.clear();
    return cudaSuccess;
}

// Kernel nodes directly in a graph (conditional bodies are separate graphs).
inline uint32_t count_kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
    uint32_t k = 0;
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

// Solver graph builder (solver.cu): appends the whole pressure solve of the
// scene's solver mode to the cursor's graph.
cudaError_t build_solve(Scene& s, GraphCursor& c);

}  // namespace apic
