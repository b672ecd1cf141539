// Host-side functions shared by the C ABI's translation units: context
// construction (xpbd_build.cu) and the rest of the ABI (xpbd_capi.cu).
#pragma once
#include "xpbd_ctx.cuh"

namespace xg {
namespace host {

// greedy vertex-disjoint colouring in item order (smallest free colour);
// entries < 0 in an item are padding. Returns the number of colours.
int greedy_colour(long long n, int arity, const int* items, long long nv, int* out);
// uploads one or more meshes and builds every device structure of a context
int build(xpbd_ctx* c, const xpbd_mesh_desc* ms, int n_inst);
// frees every device and pinned buffer of a context
void release(xpbd_ctx* c);
// positions (and the fixed flags and inverse masses in w) through the pinned
// staging buffer; returns after the upload
int stage_positions_to_device(xpbd_ctx* c, const double* x3v, const float* x3f);
// destroys the captured substep graphs (they hold buffer addresses and launch arguments)
void drop_graphs(xpbd_ctx* c);

}  // namespace host
}  // namespace xg
