// CUDA-graph capture of engine calls (declared in include/nexus_gb300.h).
//
// Every engine operation enqueues its kernels, copies and stream-ordered
// allocations (cudaMallocAsync / cudaFreeAsync of its temporaries) on the
// evaluator's or the call's stream and never waits on the host once its
// caches exist, so a sequence of calls can be recorded by stream capture and
// replayed as one graph launch.  The host-side bookkeeping of the calls
// (levels, scales, output sizes) happens while capturing; a replay repeats
// the device work on whatever the captured buffers hold, so the caller
// reloads the same input handles and reads the same output handles.
//
// Allocations the graph makes and frees (the calls' temporaries) come from
// the graph's own memory on every launch.  An output handle first sized
// inside the capture keeps a graph allocation: the graph is instantiated
// with auto-free-on-launch, so that allocation stays valid (at the same
// address) from one launch to the next, and the handle frees it as usual.
// A graph that frees memory allocated before the capture (a buffer that
// grew inside it) is refused: its second launch would free that memory
// again.  Running the calls once before capturing settles every buffer.
#include <algorithm>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/nexus_gb300.h"
#include "context.h"

struct nexus_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t nodes = 0, kernels = 0, allocs = 0, kept = 0;
};

namespace {

int fail(const char *fn, const std::string &msg)
{
    nexus::set_error(std::string(fn) + ": " + msg);
    return -1;
}

// node census; "" or the reason the graph is refused
std::string inspect(cudaGraph_t g, nexus_graph &out)
{
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return "cudaGraphGetNodes failed";
    std::vector<cudaGraphNode_t> nodes(n);
    if (n && cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return "cudaGraphGetNodes failed";
    std::vector<uintptr_t> allocated, freed;
    out.nodes = n;
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) != cudaSuccess) return "cudaGraphNodeGetType failed";
        if (t == cudaGraphNodeTypeKernel) {
            ++out.kernels;
        } else if (t == cudaGraphNodeTypeMemAlloc) {
            cudaMemAllocNodeParams p{};
            if (cudaGraphMemAllocNodeGetParams(nd, &p) != cudaSuccess) return "cudaGraphMemAllocNodeGetParams failed";
            allocated.push_back((uintptr_t)p.dptr);
        } else if (t == cudaGraphNodeTypeMemFree) {
            void *p = nullptr;
            if (cudaGraphMemFreeNodeGetParams(nd, &p) != cudaSuccess) return "cudaGraphMemFreeNodeGetParams failed";
            freed.push_back((uintptr_t)p);
        }
    }
    out.allocs = allocated.size();
    std::sort(allocated.begin(), allocated.end());
    std::sort(freed.begin(), freed.end());
    std::vector<uintptr_t> foreign;
    std::set_difference(freed.begin(), freed.end(), allocated.begin(), allocated.end(), std::back_inserter(foreign));
    if (!foreign.empty())
        return "the captured calls free " + std::to_string(foreign.size()) +
               " device buffer(s) allocated before the capture (a buffer grew inside it); run the same calls once "
               "before capturing";
    out.kept = allocated.size() - (freed.size() - foreign.size());
    return "";
}

// Refused graphs stay alive: handles that took an allocation inside the
// refused capture hold addresses reserved by that graph, which must not be
// handed out again.  Such handles are not used again (reload them first).
std::vector<cudaGraph_t> g_refused;

}  // namespace

extern "C" int nexus_graph_capture_begin(void *stream)
{
    static const char *fn = "nexus_graph_capture_begin";
    if (!stream) return fail(fn, "the legacy default stream cannot be captured: create the evaluator on a stream");
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus st;
    cudaError_t e = cudaStreamIsCapturing(s, &st);
    if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e));
    if (st != cudaStreamCaptureStatusNone) return fail(fn, "the stream is already capturing");
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e));
    return 0;
}

extern "C" int nexus_graph_capture_end(void *stream, nexus_graph **out)
{
    static const char *fn = "nexus_graph_capture_end";
    if (!stream || !out) return fail(fn, "null argument");
    *out = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        return fail(fn, std::string(cudaGetErrorString(e)) +
                            " (a captured call waited on the host or used a call that cannot be captured)");
    }
    auto *h = new nexus_graph;
    h->graph = g;
    const std::string why = inspect(g, *h);
    if (!why.empty()) {
        g_refused.push_back(g);
        delete h;
        return fail(fn, why);
    }
    e = cudaGraphInstantiate(&h->exec, g, cudaGraphInstantiateFlagAutoFreeOnLaunch);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        delete h;
        return fail(fn, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    *out = h;
    return 0;
}

extern "C" int nexus_graph_launch(const nexus_graph *g, void *stream)
{
    static const char *fn = "nexus_graph_launch";
    if (!g || !g->exec) return fail(fn, "null graph");
    cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return fail(fn, cudaGetErrorString(e));
    nexus::g_kernel_launches.fetch_add(g->kernels, std::memory_order_relaxed);
    return 0;
}

extern "C" int nexus_graph_info(const nexus_graph *g, size_t *nodes, size_t *kernel_nodes, size_t *alloc_nodes)
{
    if (!g) return fail("nexus_graph_info", "null graph");
    if (nodes) *nodes = g->nodes;
    if (kernel_nodes) *kernel_nodes = g->kernels;
    if (alloc_nodes) *alloc_nodes = g->allocs;
    return 0;
}

extern "C" int nexus_graph_destroy(nexus_graph *g)
{
    if (!g) return 0;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return 0;
}
