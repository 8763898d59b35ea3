// The whole time step as one CUDA graph (the loop body of 3D/run_3D.py:716-822 and
// 2D/run_2D.py:772-909).  The step's decisions are made on the device, so nothing waits on the
// host between phases:
//   * calc_max_speed writes max_speed to the step state and k_step_control runs the reference's
//     frame clock in double precision (curr_dt = CFL dx / max_speed, clamped to the next frame),
//     advances the step index and sets the graph's IF conditions: reinitialise this step (j == 0),
//     reseed the positions, reinitialise the flow-map gradient (k == 0);
//   * the kernels take dt from the step state (dt, dt_half), the reinitialisations run inside IF
//     nodes, and each MGPCG solve is its setup followed by a WHILE node whose body is one solver
//     iteration (the same kernels as the eager solve, so the results are bitwise the same).
// The graph is built on the first call and rebuilt only when the fields or parameters change.
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "pfm_internal.cuh"

namespace pfm {

struct StepParams {
  double CFL, dx, visualize_dt;
  int save_each, reinit_every, grad_m, repos_always, dim;
  int else_branch;  // the graph has an IF node on "not k == 0" (3D: RK4 without the gradient reinit)
};

// The frame clock (DtClock of the step loop, 3D/run_3D.py:725-743), the reinit schedule and the
// IF conditions of this step.  One thread.
__global__ void k_step_control(StepCtl* c, StepParams prm, cudaGraphConditionalHandle h_repos,
                               cudaGraphConditionalHandle h_reinit, cudaGraphConditionalHandle h_gradm,
                               cudaGraphConditionalHandle h_nogradm, unsigned long long fixed_kernels,
                               unsigned n_repos, unsigned n_reinit, unsigned n_gradm, unsigned n_nogradm) {
  const int i = c->i + 1;
  c->i = i;
  const int j = i % prm.reinit_every;
  double curr_dt = prm.CFL * prm.dx / (double)c->max_speed;
  int out = 0;
  if (prm.save_each) {
    c->frame_idx += 1;
    out = 1;
  } else if (c->sub_t + curr_dt >= prm.visualize_dt) {
    curr_dt = prm.visualize_dt - c->sub_t;
    c->sub_t = 0.0;
    c->frame_idx += 1;
    out = 1;
  } else {
    c->sub_t += curr_dt;
  }
  c->curr_dt = curr_dt;
  c->dt = (float)curr_dt;
  c->dt_half = (float)(0.5 * curr_dt);
  c->output_frame = out;
  const int reinit = j == 0;
  const int repos = reinit && (prm.repos_always || i == 0);
  // 3D restarts the gradient schedule only when it reseeds (3D/run_3D.py:753-758); 2D at every
  // reinitialisation (2D/run_2D.py:812-818)
  if (prm.dim == 3 ? repos : reinit) c->ik = i;
  const int gradm = ((i - c->ik) % prm.grad_m) == 0;
  c->reinit = reinit;
  c->repos = repos;
  c->gradm = gradm;
  cudaGraphSetConditional(h_repos, repos ? 1u : 0u);
  cudaGraphSetConditional(h_reinit, reinit ? 1u : 0u);
  cudaGraphSetConditional(h_gradm, gradm ? 1u : 0u);
  if (prm.else_branch) cudaGraphSetConditional(h_nogradm, gradm ? 0u : 1u);
  c->kernels += fixed_kernels + (repos ? n_repos : 0u) + (reinit ? n_reinit : 0u) + (gradm ? n_gradm : n_nogradm);
}

__global__ void __launch_bounds__(256) k_copy_f32(float* __restrict__ dst, const float* __restrict__ src, int64_t n) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) dst[e] = src[e];
}

__global__ void k_step_clock_set(StepCtl* c, int i, int ik, double sub_t, int frame_idx) {
  c->i = i;
  c->ik = ik;
  c->sub_t = sub_t;
  c->frame_idx = frame_idx;
}

static int copy_launch(pfm_handle* h, float* dst, const float* src, int64_t n, cudaStream_t q) {
  if (n > 0) launch(h, k_copy_f32, grid_for(n, 256), 256, 0, q, dst, src, n);
  return PFM_OK;
}

static int ensure_cap_stream(pfm_handle* h) {
  if (h->cap_stream) return PFM_OK;
  return check_cuda(h, cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking), "capture stream");
}

static int check_step_params(pfm_handle* h, const pfm_step_params* p) {
  if (!p) return set_error(h, PFM_ERR_NULL, "step: null parameters");
  if (p->reinit_every < 1 || p->reinit_every_grad_m < 1)
    return set_error(h, PFM_ERR_ARG, "step: reinit_every and reinit_every_grad_m must be >= 1");
  if (!(p->CFL > 0.0) || !(p->visualize_dt > 0.0)) return set_error(h, PFM_ERR_ARG, "step: CFL and visualize_dt must be > 0");
  if (p->poisson.max_iters < 0)
    return set_error(h, PFM_ERR_ARG, "step: the device solve needs a finite max_iters (the host does not relaunch it)");
  if (p->poisson.tol_mode < 0 || p->poisson.tol_mode > 2 || p->poisson.precision < 0 || p->poisson.precision > 2 ||
      p->poisson.warm_start < 0 || p->poisson.warm_start > 3)
    return set_error(h, PFM_ERR_ARG, "step: tol_mode and precision must be 0..2, warm_start 0..3");
  return PFM_OK;
}

static StepParams step_params(const pfm_handle* h, const pfm_step_params* p) {
  return StepParams{p->CFL, h->cfg.dx, p->visualize_dt, p->save_frame_each_step, p->reinit_every,
                    p->reinit_every_grad_m, p->reinit_particle_pos, h->cfg.dim, h->cfg.dim == 3 ? 1 : 0};
}

static int init_clock(pfm_handle* h, cudaStream_t s) {
  StepCtl* ctl = ws_ptr<StepCtl>(h, h->o_step);
  int rc = check_cuda(h, cudaMemsetAsync(ctl, 0, sizeof(StepCtl), s), "step state");
  if (rc) return rc;
  launch(h, k_step_clock_set, 1, 1, 0, s, ctl, -1, 0, 0.0, 0);
  h->step_clock_init = 1;
  return launch_check(h, "k_step_clock_set");
}

// What emitting one scene's step leaves for the finishing touch: the control kernel's node and the
// arguments it gets once the step's kernels are counted.
struct SceneEmit {
  cudaGraphNode_t ctl_node = nullptr;
  StepCtl* ctl = nullptr;
  StepParams prm{};
  cudaGraphConditionalHandle c[4] = {0, 0, 0, 0};  // reseed, reinit, k == 0, k != 0
  unsigned counts[4] = {0, 0, 0, 0};                // kernels in each IF body
  unsigned long long fixed = 0;                     // kernels outside the IF and WHILE bodies
};

// Creates the scene's IF handles in the cursor's graph, emits the step with `emit`, and counts its
// kernels.  The control kernel is captured with zero counts; patch_control sets the real ones.
template <class Emit>
static int emit_scene(GraphCursor& gc, const pfm_step_params* p, SceneEmit& se, Emit&& emit) {
  pfm_handle* h = gc.h;
  se.ctl = ws_ptr<StepCtl>(h, h->o_step);
  se.prm = step_params(h, p);
  const uint64_t before = h->launches;
  const uint64_t body0 = gc.body_launches;
  for (int k = 0; k < 4; ++k)  // one handle per IF node (a handle without a node does not instantiate)
    if (!gc.rc && (k != 3 || se.prm.else_branch))
      gc.rc = check_cuda(h, cudaGraphConditionalHandleCreate(&se.c[k], gc.G, 0, 0), "conditional handle");
  if (!gc.rc) emit(gc, se);
  gc.close();
  // the IF bodies are counted by the control kernel, the loops by the solves (on the device)
  se.fixed = (h->launches - before) - (gc.body_launches - body0);
  h->launches = before;
  return gc.rc;
}

static int patch_control(pfm_handle* h, SceneEmit& se) {
  if (!se.ctl_node) return set_error(h, PFM_ERR_CUDA, "step graph: no control node");
  cudaKernelNodeParams kp{};
  int rc = check_cuda(h, cudaGraphKernelNodeGetParams(se.ctl_node, &kp), "control node params");
  if (rc) return rc;
  void* args[] = {&se.ctl, &se.prm, &se.c[0], &se.c[1], &se.c[2], &se.c[3], &se.fixed,
                  &se.counts[0], &se.counts[1], &se.counts[2], &se.counts[3]};
  kp.kernelParams = args;
  kp.extra = nullptr;
  return check_cuda(h, cudaGraphKernelNodeSetParams(se.ctl_node, &kp), "control node params");
}

// Builds a handle's own step graph from one scene emission.
template <class Emit>
static int build_step_graph(pfm_handle* h, const pfm_step_params* p, Emit&& emit) {
  int rc = ensure_cap_stream(h);
  if (rc) return rc;
  cudaGraph_t G = nullptr;
  rc = check_cuda(h, cudaGraphCreate(&G, 0), "graph create");
  if (rc) return rc;
  GraphCursor gc(h, G, h->cap_stream);
  SceneEmit se;
  rc = emit_scene(gc, p, se, emit);
  if (!rc) rc = patch_control(h, se);
  if (h->g_step) cudaGraphExecDestroy(h->g_step);
  h->g_step = nullptr;
  if (!rc) rc = check_cuda(h, cudaGraphInstantiate(&h->g_step, G, 0), "step graph instantiate");
  cudaGraphDestroy(G);
  return rc;
}

// max_speed + control: the first segment of every scene's step; records the control kernel's node.
static void emit_head(GraphCursor& gc, SceneEmit& se, const float* u0, const float* u1, const float* u2) {
  pfm_handle* h = gc.h;
  cudaStream_t q = gc.seg();
  max_speed_async(h, u0, u1, u2, &se.ctl->max_speed, q);
  launch(h, k_step_control, 1, 1, 0, q, se.ctl, se.prm, se.c[0], se.c[1], se.c[2], se.c[3], 0ull, 0u, 0u, 0u, 0u);
  gc.close();
  se.ctl_node = gc.ndeps == 1 ? gc.deps[0] : nullptr;
}

// Kernels launched by `f` into the body of an IF node on `cond`.
template <class F>
static unsigned emit_if(GraphCursor& gc, cudaGraphConditionalHandle cond, F&& f) {
  cudaGraph_t body = gc.add_conditional(cond, cudaGraphCondTypeIf);
  if (gc.rc) return 0;
  const uint64_t b0 = gc.h->launches;
  gc.capture_body(body, [&](cudaStream_t q) { f(q); });
  return (unsigned)(gc.h->launches - b0);
}

// The step graph's key: every pointer and parameter it bakes in, member by member (no padding).
struct KeyBuf {
  std::string s;
  template <class T>
  KeyBuf& operator<<(const T& v) {
    s.append(reinterpret_cast<const char*>(&v), sizeof(T));
    return *this;
  }
};

static void key_params(KeyBuf& k, const pfm_step_params* p) {
  const pfm_solve_opts& o = p->poisson;
  k << p->CFL << p->visualize_dt << p->save_frame_each_step << p->reinit_every << p->reinit_every_grad_m
    << p->use_midpoint_vel << p->reinit_particle_pos << o.max_iters << o.eps << o.tol << o.tol_mode << o.precision
    << o.warm_start << o.true_residual_every << o.true_residual_replace;
}

static bool same_key(pfm_handle* h, const std::string& k) {
  if (h->g_step && k == h->step_key) return true;
  h->step_key = k;
  return false;
}

static int check_fields3(pfm_handle* h, const pfm3_step_fields* f, const pfm_step_params* p) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 3) return set_error(h, PFM_ERR_SHAPE, "pfm3_step on a 2D handle");
  if (!f) return set_error(h, PFM_ERR_NULL, "pfm3_step: null fields");
  int rc = check_step_params(h, p);
  if (rc) return rc;
  rc = require_ws(h);
  if (rc) return rc;
  for (int a = 0; a < 3; ++a)
    if (!f->u[a] || !f->w[a] || (p->use_midpoint_vel && !f->u_mid[a]))
      return set_error(h, PFM_ERR_NULL, "pfm3_step: null grid");
  if (!f->p) return set_error(h, PFM_ERR_NULL, "pfm3_step: null pressure");
  if (h->P > 0 && (!f->seeds || !f->pos || !f->init_imp || !f->T_init || !f->T_gm || !f->init_C))
    return set_error(h, PFM_ERR_NULL, "pfm3_step: null particle field");
  return PFM_OK;
}

static int check_fields2(pfm_handle* h, const pfm2_step_fields* f, const pfm_step_params* p) {
  if (!h) return PFM_ERR_NULL;
  if (h->cfg.dim != 2) return set_error(h, PFM_ERR_SHAPE, "pfm2_step on a 3D handle");
  if (!f) return set_error(h, PFM_ERR_NULL, "pfm2_step: null fields");
  int rc = check_step_params(h, p);
  if (rc) return rc;
  rc = require_ws(h);
  if (rc) return rc;
  for (int a = 0; a < 2; ++a)
    if (!f->u[a] || !f->w[a] || (p->use_midpoint_vel && !f->u_mid[a]))
      return set_error(h, PFM_ERR_NULL, "pfm2_step: null grid");
  if (!f->p) return set_error(h, PFM_ERR_NULL, "pfm2_step: null pressure");
  if (h->P > 0 && (!f->seeds || !f->pos || !f->imp || !f->init_imp || !f->psi || !f->T || !f->T_init || !f->T_gm ||
                   !f->init_C || !f->C))
    return set_error(h, PFM_ERR_NULL, "pfm2_step: null particle field");
  return PFM_OK;
}

static std::string key3(const pfm3_step_fields* f, const pfm_step_params* p) {
  KeyBuf key;
  key << 3;
  for (int a = 0; a < 3; ++a) key << f->u[a] << f->u_mid[a] << f->w[a];
  key << f->p << f->p_mid << f->seeds << f->pos << f->init_imp << f->T_init << f->T_gm << f->init_C;
  key_params(key, p);
  return key.s;
}

static std::string key2(const pfm2_step_fields* f, const pfm_step_params* p) {
  KeyBuf key;
  key << 2;
  for (int a = 0; a < 2; ++a) key << f->u[a] << f->u_mid[a] << f->w[a] << f->psi_grid[a];
  key << f->p << f->p_mid << f->seeds << f->pos << f->imp << f->init_imp << f->psi << f->T << f->T_init << f->T_gm
      << f->init_C << f->C;
  key_params(key, p);
  return key.s;
}

// The parts of a scene's step around its two MGPCG iteration loops: kPartAll emits the whole step
// (the loops included); a batch in work-list mode emits kPartHead (up to the midpoint solve's
// setup), kPartMid (the midpoint solve's post part up to the final solve's setup) and kPartTail
// (the final solve's post part) per scene, and the loops as batched WHILE nodes in between.
constexpr int kPartAll = -1, kPartHead = 0, kPartMid = 1, kPartTail = 2;

// One 3D step (Sim3D.step, the fused form) behind the cursor.
static void emit_step3(GraphCursor& gc, SceneEmit& se, const pfm3_step_fields* f, const pfm_step_params* p,
                       int part = kPartAll) {
  pfm_handle* h = gc.h;
  StepCtl* ctl = se.ctl;
  const bool all = part == kPartAll, mid = p->use_midpoint_vel != 0;
  const int64_t P = h->P;
  if (all || part == kPartHead) {
    emit_head(gc, se, f->u[0], f->u[1], f->u[2]);
    // j == 0: reseed (run_3D.py:753-757), G2P of the impulse, T_init = T_gm = I (:759-764)
    se.counts[0] = emit_if(gc, se.c[0], [&](cudaStream_t q) { copy_launch(h, f->pos, f->seeds, 3 * P, q); });
    se.counts[1] = emit_if(gc, se.c[1], [&](cudaStream_t q) {
      pfm3_g2p(h, f->pos, f->u[0], f->u[1], f->u[2], f->init_imp, nullptr, q);
      pfm3_reset_T(h, f->T_init, q);
      pfm3_reset_T(h, f->T_gm, q);
    });
    if (mid) {  // midpoint velocity and its projection (run_3D.py:779-788)
      launch_midpoint(h, f->u, f->u_mid, 0.f, &ctl->dt_half, gc.seg());
      append_poisson_pre(gc, f->u_mid, f->p_mid, p->poisson);
    }
  }
  if (all && mid) append_poisson_loop(gc, p->poisson, f->p_mid, ctl, 0);
  if (!(all || part == kPartMid)) {
    if (part == kPartTail) append_poisson_post(gc, f->u, f->p);
    return;
  }
  if (mid) append_poisson_post(gc, f->u_mid, f->p_mid);
  const float* ua[3] = {f->u[0], f->u[1], f->u[2]};
  if (mid)
    for (int a = 0; a < 3; ++a) ua[a] = f->u_mid[a];
  // RK4_T_forward + the P2G records, with the k == 0 gradient reinitialisation in the same kernel
  cudaMemsetAsync(ws_ptr<int>(h, h->o_count), 0, h->cells * 4, gc.seg());
  const P2GRecords3 R = records3(h, f->init_imp, f->T_init, f->init_C);
  const MacFields3 F{{ua[0], ua[1], ua[2]}}, Fg{{f->u[0], f->u[1], f->u[2]}};
  se.counts[2] = emit_if(gc, se.c[2], [&](cudaStream_t q) {
    launch_rk4_T_forward3(h, f->pos, f->T_gm, F, 0.f, &R, &Fg, q, &ctl->dt);
  });
  se.counts[3] = emit_if(gc, se.c[3], [&](cudaStream_t q) {
    launch_rk4_T_forward3(h, f->pos, f->T_gm, F, 0.f, &R, nullptr, q, &ctl->dt);
  });
  p2g3_from_records(h, f->u, f->w, gc.seg());
  append_poisson_pre(gc, f->u, f->p, p->poisson);
  if (all) {
    append_poisson_loop(gc, p->poisson, f->p, ctl, 1);
    append_poisson_post(gc, f->u, f->p);
  }
}

// One 2D step (Sim2D.step) behind the cursor (parts as emit_step3).
static void emit_step2(GraphCursor& gc, SceneEmit& se, const pfm2_step_fields* f, const pfm_step_params* p,
                       int part = kPartAll) {
  pfm_handle* h = gc.h;
  StepCtl* ctl = se.ctl;
  const bool all = part == kPartAll, mid = p->use_midpoint_vel != 0;
  const int64_t P = h->P;
  if (all || part == kPartHead) {
    emit_head(gc, se, f->u[0], f->u[1], nullptr);
    // j == 0 (2D/run_2D.py:812-832): reseed, imp = init_imp = u(pos), psi = pos, T = T_init = I
    se.counts[0] = emit_if(gc, se.c[0], [&](cudaStream_t q) { copy_launch(h, f->pos, f->seeds, 2 * P, q); });
    se.counts[1] = emit_if(gc, se.c[1], [&](cudaStream_t q) {
      pfm2_g2p(h, f->pos, f->u[0], f->u[1], f->imp, nullptr, q);
      copy_launch(h, f->init_imp, f->imp, 2 * P, q);
      copy_launch(h, f->psi, f->pos, 2 * P, q);
      pfm2_reset_T(h, f->T, q);
      pfm2_reset_T(h, f->T_init, q);
    });
    // k == 0 (2D/run_2D.py:834-843): init_C = grad u(pos), T_gm = I, T_init = T
    se.counts[2] = emit_if(gc, se.c[2], [&](cudaStream_t q) {
      pfm2_g2p(h, f->pos, f->u[0], f->u[1], nullptr, f->init_C, q);
      pfm2_reset_T(h, f->T_gm, q);
      copy_launch(h, f->T_init, f->T, 4 * P, q);
    });
    if (mid) {  // 2D/run_2D.py:866-872
      launch_midpoint(h, f->u, f->u_mid, 0.f, &ctl->dt_half, gc.seg());
      append_poisson_pre(gc, f->u_mid, f->p_mid, p->poisson);
    }
  }
  if (all && mid) append_poisson_loop(gc, p->poisson, f->p_mid, ctl, 0);
  if (!(all || part == kPartMid)) {
    if (part == kPartTail) append_poisson_post(gc, f->u, f->p);
    return;
  }
  if (mid) append_poisson_post(gc, f->u_mid, f->p_mid);
  float* ua[2] = {f->u[0], f->u[1]};
  if (mid) {
    ua[0] = f->u_mid[0];
    ua[1] = f->u_mid[1];
  }
  // RK4 of positions and T_gm, then the 2D updates and P2G (2D/run_2D.py:875-905)
  cudaStream_t q = gc.seg();
  const MacFields2 F{{ua[0], ua[1]}};
  launch_rk4_T_forward2(h, f->pos, f->T_gm, F, 0.f, 1, q, &ctl->dt);
  pfm2_update_grad_m(h, f->C, f->init_C, f->T_gm, q);
  pfm2_update_T(h, f->T, f->T_init, f->T_gm, q);
  pfm2_update_imp(h, f->imp, f->init_imp, f->T, q);
  pfm2_p2g(h, f->imp, f->pos, f->C, f->psi, f->u[0], f->u[1], f->psi_grid[0], f->psi_grid[1], f->w[0], f->w[1], q);
  append_poisson_pre(gc, f->u, f->p, p->poisson);
  if (all) {
    append_poisson_loop(gc, p->poisson, f->p, ctl, 1);
    append_poisson_post(gc, f->u, f->p);
  }
}

}  // namespace pfm

// A batch: many scenes' steps in one CUDA graph, one branch per scene (the branches share no
// data, so the graph runs them concurrently).
struct pfm_batch {
  struct Scene {
    pfm_handle* h;
    int dim;
    pfm3_step_fields f3;
    pfm2_step_fields f2;
    pfm_step_params p;
  };
  std::vector<Scene> scenes;
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  int valid = 0;
  int worklist = 0;  // 1: the scenes' MGPCG iterations run as batched work-list kernels
  std::string err;
};

namespace pfm {

static bool same_solve(const pfm_step_params& a, const pfm_step_params& b) {
  const pfm_solve_opts &x = a.poisson, &y = b.poisson;
  return a.use_midpoint_vel == b.use_midpoint_vel && x.max_iters == y.max_iters && x.eps == y.eps &&
         x.tol == y.tol && x.tol_mode == y.tol_mode && x.precision == y.precision &&
         x.true_residual_every == y.true_residual_every && x.true_residual_replace == y.true_residual_replace;
}

// Work-list form of a batch step: every scene's step runs in its own branch up to the setup of a
// solve, the branches join, one WHILE node advances every scene's MGPCG iterations with batched
// work-list kernels (each kernel of the iteration one launch for all scenes, work items = the
// scenes' own thread blocks; a scene whose solve has converged skips its items), and the branches
// fork again behind it.  Each scene's kernels run in their own order on their own data, so the
// results are bitwise those of stepping the scenes alone.
static int build_batch_worklist(pfm_batch* b, cudaGraph_t G) {
  const size_t n = b->scenes.size();
  const pfm_batch::Scene& s0 = b->scenes[0];
  if (n > 128) {
    b->err = "work-list batch: at most 128 scenes";
    return PFM_ERR_ARG;
  }
  for (const auto& sc : b->scenes) {
    if (sc.dim != s0.dim || !same_solve(sc.p, s0.p)) {
      b->err = "work-list batch: the scenes must share the dimension, the midpoint flag and the solver options";
      return PFM_ERR_ARG;
    }
    if (sc.h->smooth_tma) {
      b->err = "work-list batch: the TMA-staged smoother is not batched (tuning key PFM_TUNE_SMOOTH_TMA = 0)";
      return PFM_ERR_ARG;
    }
  }
  std::vector<std::unique_ptr<GraphCursor>> cur;
  std::vector<SceneEmit> se(n);
  std::vector<uint64_t> before(n);
  std::vector<pfm_handle*> hs(n);
  std::vector<StepCtl*> ctls(n);
  for (size_t s = 0; s < n; ++s) {
    const auto& sc = b->scenes[s];
    hs[s] = sc.h;
    cur.emplace_back(new GraphCursor(sc.h, G, b->cap));
    se[s].ctl = ws_ptr<StepCtl>(sc.h, sc.h->o_step);
    se[s].prm = step_params(sc.h, &sc.p);
    ctls[s] = se[s].ctl;
    before[s] = sc.h->launches;
    GraphCursor& gc = *cur[s];
    for (int k = 0; k < 4; ++k)
      if (!gc.rc && (k != 3 || se[s].prm.else_branch))
        gc.rc = check_cuda(sc.h, cudaGraphConditionalHandleCreate(&se[s].c[k], G, 0, 0), "conditional handle");
    if (gc.rc) {
      b->err = sc.h->err;
      return gc.rc;
    }
  }
  auto emit_part = [&](int part) -> int {
    for (size_t s = 0; s < n; ++s) {
      const auto& sc = b->scenes[s];
      GraphCursor& gc = *cur[s];
      if (sc.dim == 3)
        emit_step3(gc, se[s], &sc.f3, &sc.p, part);
      else
        emit_step2(gc, se[s], &sc.f2, &sc.p, part);
      gc.close();
      if (gc.rc) {
        b->err = sc.h->err;
        return gc.rc;
      }
    }
    return PFM_OK;
  };
  uint64_t joint_body = 0;  // batched body kernels: counted on the device, not as fixed kernels
  auto batched = [&](int which) -> int {
    GraphCursor J(hs[0], G, b->cap);
    J.ndeps = 0;
    for (size_t s = 0; s < n; ++s)
      for (size_t d = 0; d < cur[s]->ndeps; ++d) {
        if (J.ndeps == sizeof(J.deps) / sizeof(J.deps[0])) {
          b->err = "work-list batch: too many branch ends to join";
          return PFM_ERR_ARG;
        }
        J.deps[J.ndeps++] = cur[s]->deps[d];
      }
    int rc = append_batched_loop(J, hs.data(), (int)n, s0.p.poisson, ctls.data(), which);
    J.close();
    if (!rc) rc = J.rc;
    if (rc) {
      b->err = hs[0]->err;
      return rc;
    }
    joint_body += J.body_launches;
    for (size_t s = 0; s < n; ++s) {  // fork: each scene's finish and statistics, then its next part
      const auto& sc = b->scenes[s];
      GraphCursor& gc = *cur[s];
      gc.ndeps = J.ndeps;
      for (size_t d = 0; d < J.ndeps; ++d) gc.deps[d] = J.deps[d];
      float* p_io = which == 0 ? (sc.dim == 3 ? sc.f3.p_mid : sc.f2.p_mid) : (sc.dim == 3 ? sc.f3.p : sc.f2.p);
      append_poisson_finish(gc, sc.p.poisson, p_io, ctls[s], which);
      gc.close();  // the branches share one capture stream: one open segment at a time
      if (gc.rc) {
        b->err = sc.h->err;
        return gc.rc;
      }
    }
    return PFM_OK;
  };
  int rc = emit_part(kPartHead);
  if (!rc && s0.p.use_midpoint_vel) rc = batched(0);
  if (!rc) rc = emit_part(kPartMid);
  if (!rc) rc = batched(1);
  if (!rc) rc = emit_part(kPartTail);
  if (rc) return rc;
  for (size_t s = 0; s < n; ++s) {
    const auto& sc = b->scenes[s];
    GraphCursor& gc = *cur[s];
    gc.close();
    se[s].fixed = (sc.h->launches - before[s]) - gc.body_launches - (s == 0 ? joint_body : 0);
    sc.h->launches = before[s];
    rc = patch_control(sc.h, se[s]);
    if (rc) {
      b->err = sc.h->err;
      return rc;
    }
    if (sc.dim == 3) sc.h->rec_valid = 1;
  }
  return PFM_OK;
}

}  // namespace pfm

using namespace pfm;

extern "C" {

int pfm3_step(pfm_handle* h, const pfm3_step_fields* f, const pfm_step_params* p, void* stream) {
  int rc = check_fields3(h, f, p);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (!h->step_clock_init) {
    rc = init_clock(h, s);
    if (rc) return rc;
  }
  if (!same_key(h, key3(f, p))) {
    rc = build_step_graph(h, p, [&](GraphCursor& gc, SceneEmit& se) { emit_step3(gc, se, f, p); });
    if (rc) {
      h->step_key.clear();
      return rc;
    }
    h->rec_valid = 1;
  }
  return check_cuda(h, cudaGraphLaunch(h->g_step, s), "step graph launch");
}

int pfm2_step(pfm_handle* h, const pfm2_step_fields* f, const pfm_step_params* p, void* stream) {
  int rc = check_fields2(h, f, p);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (!h->step_clock_init) {
    rc = init_clock(h, s);
    if (rc) return rc;
  }
  if (!same_key(h, key2(f, p))) {
    rc = build_step_graph(h, p, [&](GraphCursor& gc, SceneEmit& se) { emit_step2(gc, se, f, p); });
    if (rc) {
      h->step_key.clear();
      return rc;
    }
  }
  return check_cuda(h, cudaGraphLaunch(h->g_step, s), "step graph launch");
}

int pfm_batch_create(pfm_batch** out) {
  if (!out) return PFM_ERR_NULL;
  *out = new (std::nothrow) pfm_batch();
  return *out ? PFM_OK : PFM_ERR_CUDA;
}

int pfm_batch_destroy(pfm_batch* b) {
  if (!b) return PFM_ERR_NULL;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->cap) cudaStreamDestroy(b->cap);
  delete b;
  return PFM_OK;
}

const char* pfm_batch_last_error(const pfm_batch* b) { return b ? b->err.c_str() : "null batch"; }

int pfm_batch_set_worklist(pfm_batch* b, int on) {
  if (!b) return PFM_ERR_NULL;
  if (on != 0 && on != 1) {
    b->err = "pfm_batch_set_worklist: on must be 0 or 1";
    return PFM_ERR_ARG;
  }
  if (b->worklist != on) b->valid = 0;
  b->worklist = on;
  return PFM_OK;
}

static int batch_add(pfm_batch* b, pfm_handle* h, int dim, const pfm3_step_fields* f3, const pfm2_step_fields* f2,
                     const pfm_step_params* p) {
  if (!b || !h || !p) return PFM_ERR_NULL;
  for (const auto& sc : b->scenes)
    if (sc.h == h) {
      b->err = "pfm_batch_add: a handle can be in a batch once (its workspace holds the scene's state)";
      return PFM_ERR_ARG;
    }
  int rc = dim == 3 ? check_fields3(h, f3, p) : check_fields2(h, f2, p);
  if (rc) {
    b->err = std::string("pfm_batch_add: ") + h->err;
    return rc;
  }
  pfm_batch::Scene sc{};
  sc.h = h;
  sc.dim = dim;
  if (f3) sc.f3 = *f3;
  if (f2) sc.f2 = *f2;
  sc.p = *p;
  b->scenes.push_back(sc);
  b->valid = 0;
  return PFM_OK;
}

int pfm_batch_add3(pfm_batch* b, pfm_handle* h, const pfm3_step_fields* f, const pfm_step_params* p) {
  return batch_add(b, h, 3, f, nullptr, p);
}

int pfm_batch_add2(pfm_batch* b, pfm_handle* h, const pfm2_step_fields* f, const pfm_step_params* p) {
  return batch_add(b, h, 2, nullptr, f, p);
}

int pfm_batch_step(pfm_batch* b, void* stream) {
  if (!b) return PFM_ERR_NULL;
  if (b->scenes.empty()) {
    b->err = "pfm_batch_step: empty batch";
    return PFM_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  for (auto& sc : b->scenes)
    if (!sc.h->step_clock_init) {
      int rc = init_clock(sc.h, s);
      if (rc) {
        b->err = sc.h->err;
        return rc;
      }
    }
  if (!b->valid) {
    if (!b->cap) {
      cudaError_t e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
      if (e != cudaSuccess) {
        b->err = std::string("capture stream: ") + cudaGetErrorString(e);
        return PFM_ERR_CUDA;
      }
    }
    cudaGraph_t G = nullptr;
    if (cudaGraphCreate(&G, 0) != cudaSuccess) {
      b->err = "graph create failed";
      return PFM_ERR_CUDA;
    }
    int rc = PFM_OK;
    if (b->worklist) rc = build_batch_worklist(b, G);
    for (auto& sc : b->scenes) {  // every scene a branch from the graph's roots
      if (b->worklist) break;
      GraphCursor gc(sc.h, G, b->cap);
      SceneEmit se;
      if (sc.dim == 3)
        rc = emit_scene(gc, &sc.p, se, [&](GraphCursor& g, SceneEmit& e) { emit_step3(g, e, &sc.f3, &sc.p); });
      else
        rc = emit_scene(gc, &sc.p, se, [&](GraphCursor& g, SceneEmit& e) { emit_step2(g, e, &sc.f2, &sc.p); });
      if (!rc) rc = patch_control(sc.h, se);
      if (rc) {
        b->err = sc.h->err;
        break;
      }
      if (sc.dim == 3) sc.h->rec_valid = 1;
    }
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    if (!rc) {
      cudaError_t e = cudaGraphInstantiate(&b->exec, G, 0);
      if (e != cudaSuccess) {
        b->err = std::string("batch graph instantiate: ") + cudaGetErrorString(e);
        rc = PFM_ERR_CUDA;
      }
    }
    cudaGraphDestroy(G);
    if (rc) return rc;
    b->valid = 1;
  }
  const cudaError_t e = cudaGraphLaunch(b->exec, s);
  if (e != cudaSuccess) {
    b->err = std::string("batch graph launch: ") + cudaGetErrorString(e);
    return PFM_ERR_CUDA;
  }
  return PFM_OK;
}

int pfm_step_reset(pfm_handle* h, int i, int ik, double sub_t, int frame_idx, void* stream) {
  if (!h) return PFM_ERR_NULL;
  int rc = require_ws(h);
  if (rc) return rc;
  StepCtl* ctl = ws_ptr<StepCtl>(h, h->o_step);
  cudaStream_t s = (cudaStream_t)stream;
  rc = check_cuda(h, cudaMemsetAsync(ctl, 0, sizeof(StepCtl), s), "step state");
  if (rc) return rc;
  launch(h, k_step_clock_set, 1, 1, 0, s, ctl, i, ik, sub_t, frame_idx);
  h->step_clock_init = 1;
  return launch_check(h, "k_step_clock_set");
}

int pfm_reset_warm_history(pfm_handle* h, void* stream) {
  if (!h) return PFM_ERR_NULL;
  int rc = require_ws(h);
  if (rc) return rc;
  return check_cuda(h, cudaMemsetAsync(ws_ptr<int>(h, h->o_hist_flag), 0, 2 * sizeof(int), (cudaStream_t)stream),
                    "pressure history flags");
}

int pfm_step_info(pfm_handle* h, pfm_step_info_t* info, void* stream) {
  if (!h || !info) return PFM_ERR_NULL;
  int rc = require_ws(h);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  StepCtl c;
  StepCtl* ctl = ws_ptr<StepCtl>(h, h->o_step);
  rc = check_cuda(h, cudaMemcpyAsync(&c, ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, s), "step state read");
  if (!rc) rc = check_cuda(h, cudaStreamSynchronize(s), "step state sync");
  if (!rc) rc = check_cuda(h, cudaMemsetAsync(&ctl->kernels, 0, sizeof(ctl->kernels), s), "step kernel count");
  if (rc) return rc;
  h->launches += c.kernels;
  info->step = c.i;
  info->ik = c.ik;
  info->frame_idx = c.frame_idx;
  info->output_frame = c.output_frame;
  info->reinit = c.reinit;
  info->reseed = c.repos;
  info->gradm_reinit = c.gradm;
  info->dt = c.curr_dt;
  info->sub_t = c.sub_t;
  info->max_speed = c.max_speed;
  for (int k = 0; k < 2; ++k) {
    info->iterations[k] = c.iters[k];
    info->converged[k] = c.done[k] == 1;
    info->rTr[k] = c.rTr[k];
  }
  for (int k = 0; k < 64; ++k) {
    info->history[k][0] = c.history[k][0];
    info->history[k][1] = c.history[k][1];
  }
  return PFM_OK;
}

}  // extern "C"
