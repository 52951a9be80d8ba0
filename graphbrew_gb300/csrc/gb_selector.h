// gb_selector.h -- Tier-0 features and the learned selector's MLP (selector.cu).
#pragma once

#include "gb_common.cuh"

namespace gb {

constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 3;   // arms: GraphBrew algorithm 12, DBG, original order

// out[0..8] = num_nodes, num_edges (directed), avg_degree, degree_cv,
// internal_density, hub_concentration, packing_factor, normalized_edge_span,
// window_neighbor_overlap.
void tier0_features_device(const DeviceCSR& g, double* out9_host, cudaStream_t s);

int mlp_param_count(int in_dim);
// Y[B x 3] = MLP(X[B x in]); H1/H2 are B x 64 activations (device).
void mlp_forward_device(const float* params, const float* X, int B, int in, float* Y, float* H1, float* H2,
                        cudaStream_t s);
// Mean squared error of MLP(X) against T and its gradient (same layout as params).
float mlp_grad_device(const float* params, const float* X, const float* T, int B, int in, float* grad,
                      cudaStream_t s);
// Adam on shuffled minibatches; params updated in place; returns the last epoch's mean loss.
float mlp_train_device(float* params, const float* X, const float* T, int n, int in, int epochs, int batch,
                       float lr, uint64_t seed, cudaStream_t s);

}  // namespace gb
