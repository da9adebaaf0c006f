// Sampler workspaces and host orchestration (internal).
#pragma once
#include <stdint.h>

#include <map>
#include <vector>

#include "engine.h"

namespace gbm {

// Per-chain flags (one byte per chain).
enum ChainFlag : uint8_t {
  kCont = 1,        // trajectory still growing (continue_tree)
  kNotDiv = 2,      // no divergence so far (not_divergence)
  kAccepted = 4,    // a new candidate was chosen (is_accepted)
  kSubCont = 8,     // current subtree still growing
  kSubNotDiv = 16,  // subtree-level not_divergence
  kForward = 32,    // direction of the current subtree
  kRunning = 64,    // free-running loop: the chain has transitions left
};

// Free-running NUTS (every chain at its own transition, depth and leaf):
// per-chain loop state on the device.
enum FreePhase : uint8_t { kPhaseStart = 0, kPhaseDepth = 1, kPhaseLeaf = 2 };

struct FreeDev {
  int* t;                   // [C] transitions completed
  int* depth;               // [C] tree depth of the current doubling
  int* leaf;                // [C] leaf within the current subtree
  uint8_t* phase;           // [C] FreePhase
  uint2* key;               // [C] key of the current transition
  const int* wtab;          // [2^max_depth] write slot per leaf (-1: none)
  const int* rlo;           // [2^max_depth] U-turn read range per leaf
  const int* rhi;
  const float* eps_in;      // step size: [1] or [C]
  int eps_per_chain;
  uint2 seed;
  uint32_t first;           // sample_chain step of each chain's transition 0
  int kmax;                 // transitions per chain
  int max_depth;
  double max_energy_diff;
  // Trace [kmax][...]; any may be NULL.
  float* tr_state;          // [kmax][state elements]
  double* tr_logp;          // [kmax][C]
  double* tr_lar;
  int32_t* tr_lf;
  uint8_t* tr_acc;
  uint8_t* tr_div;
  // Streaming moments (Welford, float64 [C][D]) of each chain's results:
  // transition t of a chain is draw mom_base + t of its running mean / M2.
  double* mom_mean;
  double* mom_m2;
  int64_t mom_base;
  size_t tr_estride;        // state elements per transition
};

// Device pointers of the NUTS workspace (passed to kernels by value).
// Uniform layout: chain c's D-vector starts at c * D.  Ragged layout (many
// posteriors of different dimension in one sampler): chain c's vector has
// cdim[c] elements starting at coff[c], its U-turn slots start at
// coff[c] * slots, and the gradient batch is evaluated in place (qw, gw at
// coff[c], lw[c]) instead of compacted.
struct NutsDev {
  int C, D, slots;
  int ragged;
  const int64_t* coff;      // [C] element offsets (ragged)
  const int* cdim;          // [C] dimensions (ragged)
  // Diagonal inverse mass matrix (PreconditionedNoUTurnSampler): NULL for
  // the identity, else [D] shared by every chain or, with im_per_chain, one
  // entry per state element (the layout of the states).
  const float* inv_mass;
  int im_per_chain;
  float* end_q[2];
  float* end_p[2];
  float* end_g[2];
  double* end_l[2];
  float *cand_q, *cand_g, *sub_q, *sub_g, *mom_sum, *cumsum;
  float *slot_p, *slot_cs;  // [C][slots][D]
  float *qw, *gw;           // compacted batch [C][D]
  double* lw;               // [C]
  double *cand_l, *cand_e, *cand_w, *sub_l, *sub_e, *sub_w, *e0, *eds, *sub_eds;
  int *lf, *sub_lf, *tree_depth;
  uint8_t* flags;
  float* eps;               // |step size| per chain
  int* act_idx;             // [C]
  int* act_count;           // [1]
  int* act_blk;             // [ceil(C / 1024)] per-block counts of the compaction
  int* any_cont;            // [1]
};

struct NutsOutputs {
  float* state;
  double* target_log_prob;
  float* grads;
  double* log_accept_ratio;
  int32_t* leapfrogs_taken;
  uint8_t* is_accepted;
  uint8_t* reach_max_depth;
  uint8_t* has_divergence;
  double* energy;
  int32_t* tree_depth;      // optional
};

struct HmcOutputs {
  float* next_state;
  double* next_tlp;
  float* next_grads;
  float* proposed_state;
  double* proposed_tlp;
  float* proposed_grads;
  float* initial_momentum;
  float* final_momentum;
  double* log_acceptance_correction;
  double* log_accept_ratio;
  uint8_t* is_accepted;
};

struct DaParams {
  double target_accept_prob, exploration_shrinkage, step_count_smoothing, decay_rate;
  int num_adaptation_steps;
};

// Traced outputs of a device-resident chain loop; any pointer may be NULL.
struct ChainTrace {
  float* state;               // [R][C][D]
  double* target_log_prob;    // [R][C]
  double* log_accept_ratio;   // [R][C]
  int32_t* leapfrogs_taken;   // [R][C] (NUTS)
  uint8_t* is_accepted;       // [R][C]
  uint8_t* has_divergence;    // [R][C] (NUTS)
  float* step_size;           // [R][groups]
  // Streaming moments of the traced states (Welford, float64 [C][D]): the
  // per-chain running mean and sum of squared deviations over the results,
  // for diagnostics without storing the draws.
  double* moment_mean;
  double* moment_m2;
};

// Fold one state [n elements] into running moments after `count_before`
// earlier samples (Welford).
void autocov_update(cudaStream_t s, const float* x, size_t E, int64_t count_before, int L,
                    float* x0, double* total, float* head, float* ring, double* lag);
void moments_update(cudaStream_t s, const float* x, size_t n, int64_t count_before, double* mean,
                    double* m2);

// Dual-averaging configuration of a chain loop (enabled = 0: fixed step).
struct DaConfig {
  int enabled;
  DaParams prm;
  const double* target_accept;  // [groups] or NULL
  double* state;                // [groups][4]
};

}  // namespace gbm

struct gbm_nuts;
struct gbm_hmc;

namespace gbm {
void nuts_setup(gbm_nuts* k);
void nuts_one_step(gbm_nuts* k, int64_t chains, const float* q, const double* l, const float* g,
                   const float* eps, int eps_per_chain, uint2 key, const NutsOutputs& out);
void hmc_setup(gbm_hmc* k);
// Launches of one HMC transition with the key read from device memory.
void hmc_step_launches(gbm_hmc* k, int64_t chains, const float* q, const double* l,
                       const float* g, const float* eps, int per_chain, int num_leapfrog_steps,
                       const uint2* keyp, const HmcOutputs& out, cudaStream_t s);
void hmc_one_step(gbm_hmc* k, int64_t chains, const float* q, const double* l, const float* g,
                  const float* eps, int per_chain, int num_leapfrog_steps, uint2 key,
                  const HmcOutputs& out);
void metropolis_hastings_step(cudaStream_t s, int64_t C, int64_t D, uint2 key,
                              const double* cur_tlp, const double* prop_tlp, const double* corr,
                              const float* cur_q, const float* prop_q, float* next_q,
                              double* lar, uint8_t* acc);
void dual_averaging_update_reduced(cudaStream_t s, const double* reduced, int64_t groups,
                                   const DaParams& prm, const double* target_accept,
                                   double* state, float* eps);
void dual_averaging_update(cudaStream_t s, const double* lar, int64_t C, int per_chain,
                           const DaParams& prm, const double* target_accept, double* state,
                           float* eps);
// Free-running NUTS: each chain runs `kmax` transitions (keys step_key(seed,
// first_step + t)) and starts its next transition as soon as its own tree
// ends, so one long trajectory does not hold the others; at most
// `max_leaf_iterations` leaf iterations.  Writes the trace and, per chain,
// the transitions completed; returns the leaf iterations run.
int64_t nuts_run_free(gbm_nuts* k, int64_t C, const float* q, const double* l, const float* g,
                      const float* eps, int eps_per_chain, uint2 seed, uint32_t first_step,
                      int kmax, int64_t max_leaf_iterations, FreeDev trace,
                      int32_t* transitions_done);
void nuts_sample_chain(gbm_nuts* k, int64_t C, float* q, double* l, float* g, float* eps,
                       int per_chain, uint2 seed, uint32_t first_step, int64_t num_results,
                       int64_t burnin, int64_t thin, const DaConfig& da, const ChainTrace& tr);
void hmc_sample_chain(gbm_hmc* k, int64_t C, float* q, double* l, float* g, float* eps,
                      int per_chain, int num_leapfrog_steps, uint2 seed, uint32_t first_step,
                      int64_t num_results, int64_t burnin, int64_t thin, const DaConfig& da,
                      const ChainTrace& tr);
}  // namespace gbm

struct gbm_nuts {
  gbm_target* target = nullptr;   // must outlive every call except destroy
  gbm_context* ctx = nullptr;
  int64_t max_chains = 0;
  int max_tree_depth = 10;
  double max_energy_diff = 1000.0;
  int unrolled_leapfrog_steps = 1;
  std::vector<int> write_instr;             // per leaf (dummy = -1)
  std::vector<int> read_lo, read_hi;        // per leaf
  gbm::DeviceBuffer mem;
  gbm::DeviceBuffer target_ws;
  gbm::DeviceBuffer loop_mem;   // chain-loop ping-pong and result buffers
  gbm::NutsDev dev{};
  cudaEvent_t poll_events[4] = {nullptr, nullptr, nullptr, nullptr};
  // CUDA-graph replay of batches of leaves (ragged batches on a non-default
  // stream): one executable graph per (depth, first leaf), captured on first
  // use; the transition key is read from key_dev so graphs are reused by
  // every transition.
  bool use_graphs = false;
  const float* inv_mass = nullptr;   // see NutsDev
  int im_per_chain = 0;
  cudaStream_t graph_stream = nullptr;   // capture stream (graphs launch on the caller's)
  std::map<int64_t, cudaGraphExec_t> graphs;   // (chains, depth, first leaf)
  gbm::DeviceBuffer key_dev;   // uint2
  gbm::DeviceBuffer free_mem;  // free-running loop: per-chain state and leaf tables
  // sample_chain runs the draws after adaptation (fixed step size, no
  // thinning) free-running: per chain the same transitions, without waiting
  // for the batch's longest trajectory.
  bool free_draws = false;
  gbm::DeviceBuffer free_lar;  // log-accept ratios of a free segment when none are traced
  int64_t graph_launches = 0;
  // Counters for the last transition (host-visible after one_step returns).
  int64_t last_leaf_iterations = 0;
  // Optional profiling: CUDA events bracket every batched target evaluation.
  bool profiling = false;
  std::vector<cudaEvent_t> prof_events;  // pairs (start, end)
  size_t prof_used = 0;                  // events recorded since the last flush
  double prof_eval_ms = 0.0;
  int64_t prof_evals = 0;
  int64_t prof_launches = 0;             // every kernel this handle launched
};

namespace gbm {
void nuts_profile_flush(gbm_nuts* k);  // stream must be synchronized
void nuts_release_graphs(gbm_nuts* k);
void nuts_clear_graphs(gbm_nuts* k);   // keep the capture stream
}  // namespace gbm

struct gbm_hmc {
  gbm_target* target = nullptr;   // must outlive every call except destroy
  gbm_context* ctx = nullptr;
  int64_t max_chains = 0;
  gbm::DeviceBuffer mem;
  gbm::DeviceBuffer target_ws;
  gbm::DeviceBuffer loop_mem;   // chain-loop ping-pong and result buffers
  gbm::DeviceBuffer key_dev;    // uint2 transition key + uint32 step counter
  bool use_graphs = true;       // device loops replay each transition as a graph
};
