// The GPU operators inside the reference tree. Compiled with
// QEG_WITH_REFERENCE_HEADERS against the reference's own headers and linked
// with the reference engine (built from its sources) and libqeg.so, this
// program lowers plans from the reference's own plan generator
// (oracle::gen_plan_case, oracle/generators.h:196) twice:
//   * the reference's Plan::lower (plan/plan.cpp:581-614), and
//   * lower_gpu() below: the same tree with every Aggregate, Join, tumbling
//     Window and AsofJoin node replaced by its GPU operator -- the lowering
//     switch a maintainer adds to Plan::lower.
// Both trees are drained with the reference's oracle::drain_operator and
// compared with its compare_result_sets (oracle/result_set.h:59-75; unordered,
// because a GPU aggregate emits its groups in another order and a Sort above
// it may order ties differently). Without a CUDA device the GPU trees are
// built but not run, and the program says so; exit code 0 = every check
// passed.
#include <cstdio>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>

#include "oracle/generators.h"
#include "oracle/result_set.h"
#include "ops/filter.h"
#include "ops/project.h"
#include "ops/sort.h"
#include "plan/plan.h"
#include "query-engine_gb300/host/gpu_operators.h"
#include "tsx/asof.h"
#include "tsx/window.h"

using namespace qe;

namespace {

// Plan::lower with the GPU operators for the hash-table nodes.
std::unique_ptr<Operator> lower_gpu(const plan::Plan& p, std::size_t batch) {
  const plan::PlanNode& n = p.node();
  switch (n.kind) {
    case plan::PlanKind::Aggregate:
      return std::make_unique<gpu::GpuAggregate>(lower_gpu(n.children[0], batch), n.group_keys, n.aggs);
    case plan::PlanKind::Join:
      return std::make_unique<gpu::GpuHashJoin>(lower_gpu(n.children[0], batch), lower_gpu(n.children[1], batch),
                                                n.left_keys, n.right_keys, n.join_type);
    case plan::PlanKind::AsofJoin:
      return std::make_unique<gpu::GpuAsofJoin>(lower_gpu(n.children[0], batch), lower_gpu(n.children[1], batch),
                                                n.asof_left_keys, n.asof_right_keys, n.asof_left_time,
                                                n.asof_right_time, n.asof_type, n.asof_tolerance);
    case plan::PlanKind::Window:
      if (n.window_mode == tsx::WindowMode::Tumbling)
        return std::make_unique<gpu::GpuWindow>(lower_gpu(n.children[0], batch), n.window_mode, n.window_keys,
                                                n.window_time, n.window_param, n.window_aggs);
      return std::make_unique<tsx::Window>(lower_gpu(n.children[0], batch), n.window_mode, n.window_keys,
                                           n.window_time, n.window_param, n.window_aggs);
    case plan::PlanKind::Filter:
      return std::make_unique<Filter>(lower_gpu(n.children[0], batch), n.predicate);
    case plan::PlanKind::Project:
      return std::make_unique<Project>(lower_gpu(n.children[0], batch), n.projections);
    case plan::PlanKind::Sort:
      return std::make_unique<Sort>(lower_gpu(n.children[0], batch), n.sort_keys);
    default:  // leaves (Scan, CompressedScan)
      return p.lower(batch);
  }
}

int count_gpu_nodes(const plan::Plan& p) {
  const plan::PlanNode& n = p.node();
  int c = (n.kind == plan::PlanKind::Aggregate || n.kind == plan::PlanKind::Join ||
           n.kind == plan::PlanKind::AsofJoin ||
           (n.kind == plan::PlanKind::Window && n.window_mode == tsx::WindowMode::Tumbling))
              ? 1
              : 0;
  for (const plan::Plan& ch : n.children) c += count_gpu_nodes(ch);
  return c;
}

bool have_gpu() {
  qeg_ctx* ctx = nullptr;
  if (qeg_ctx_create(0, &ctx) != QEG_OK) return false;
  qeg_ctx_destroy(ctx);
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  const int cases = argc > 1 ? std::atoi(argv[1]) : 60;
  const bool gpu = have_gpu();
  if (!gpu) std::printf("no CUDA device: GPU trees are built but not run\n");
  int fails = 0, compared = 0, gpu_nodes = 0;
  for (int i = 0; i < cases; ++i) {
    std::mt19937_64 rng(0x9E3779B9ull * (i + 1));
    oracle::PlanCase pc = oracle::gen_plan_case(rng);
    const std::size_t batch = (i % 3 == 0) ? 64 : 2048;
    std::unique_ptr<Operator> cpu_tree = pc.plan.lower(batch);
    std::unique_ptr<Operator> gpu_tree;
    try {
      gpu_tree = lower_gpu(pc.plan, batch);
    } catch (const std::invalid_argument& e) {
      // A node the GPU operators reject at construction (out of their grammar)
      // must be rejected by the reference too, or be outside the hot path.
      std::printf("case %d: GPU lowering rejected the plan: %s\n", i, e.what());
      continue;
    }
    gpu_nodes += count_gpu_nodes(pc.plan);
    // The trees expose the same schema.
    const Schema a = cpu_tree->output_schema(), b = gpu_tree->output_schema();
    bool same = a.fields.size() == b.fields.size();
    for (std::size_t c = 0; same && c < a.fields.size(); ++c) same = a.fields[c].second == b.fields[c].second;
    if (!same) {
      std::printf("case %d: output schemas differ\n%s\n", i, pc.plan.to_string().c_str());
      ++fails;
      continue;
    }
    const oracle::ResultSet want = oracle::drain_operator(*cpu_tree);
    if (!gpu) continue;
    const oracle::ResultSet got = oracle::drain_operator(*gpu_tree);
    const oracle::DiffResult d = oracle::compare_result_sets(got, want, false);
    ++compared;
    if (!d.equal) {
      std::printf("case %d differs: %s\n%s\n", i, d.message.c_str(), pc.plan.to_string().c_str());
      ++fails;
    }
  }
  std::printf("%d plans, %d GPU nodes, %d compared on the GPU, %d failures\n", cases, gpu_nodes, compared, fails);
  return fails ? 1 : 0;
}
