// capi.cu -- ABI version and the per-thread error message.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "capi_util.h"

namespace {
thread_local char g_error[512] = "";
}

namespace d3d {
void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}
}  // namespace d3d

extern "C" int d3d_abi_version(void) { return D3D_ABI_VERSION; }

namespace {

// Kernel nodes of a graph and of its child graphs, split by where the kernel
// comes from: this library's own kernels, or the CUDA toolkit's CUB templates
// the library instantiates (their mangled names carry the cub namespace).
// Kernels whose name the runtime cannot give count as neither.
cudaError_t count_kernels(cudaGraph_t g, int64_t* own, int64_t* toolkit, int depth) {
    size_t n = 0;
    cudaError_t e = cudaGraphGetNodes(g, nullptr, &n);
    if (e != cudaSuccess || n == 0) return e;
    cudaGraphNode_t* nodes = static_cast<cudaGraphNode_t*>(malloc(n * sizeof(cudaGraphNode_t)));
    if (!nodes) return cudaErrorMemoryAllocation;
    e = cudaGraphGetNodes(g, nodes, &n);
    for (size_t k = 0; e == cudaSuccess && k < n; ++k) {
        cudaGraphNodeType t;
        e = cudaGraphNodeGetType(nodes[k], &t);
        if (e != cudaSuccess) break;
        if (t == cudaGraphNodeTypeKernel) {
            cudaKernelNodeParams p = {};
            const char* name = nullptr;
            cudaError_t q = cudaGraphKernelNodeGetParams(nodes[k], &p);
            if (q == cudaSuccess && p.func) q = cudaFuncGetName(&name, p.func);
            if (q == cudaSuccess && name) {
                if (strstr(name, "3cub") || strstr(name, "cub::"))
                    ++*toolkit;
                else
                    ++*own;
            } else if (q != cudaSuccess) {
                cudaGetLastError();  // a kernel the runtime cannot name leaves no error behind
            }
        } else if (t == cudaGraphNodeTypeGraph && depth < 8) {
            cudaGraph_t child;
            e = cudaGraphChildGraphNodeGetGraph(nodes[k], &child);
            if (e == cudaSuccess) e = count_kernels(child, own, toolkit, depth + 1);
        }
    }
    free(nodes);
    return e;
}

}  // namespace

extern "C" int d3d_graph_kernel_nodes(const void* graph, int64_t* own, int64_t* toolkit) {
    D3D_REQUIRE(graph && own && toolkit, "d3d_graph_kernel_nodes: null argument");
    *own = *toolkit = 0;
    cudaGraph_t g = reinterpret_cast<cudaGraph_t>(const_cast<void*>(graph));
    const cudaError_t e = count_kernels(g, own, toolkit, 0);
    if (e != cudaSuccess) {
        d3d::set_error("d3d_graph_kernel_nodes: %s", cudaGetErrorString(e));
        return D3D_ERR_CUDA;
    }
    return D3D_SUCCESS;
}

extern "C" const char* d3d_last_error(void) { return g_error; }
