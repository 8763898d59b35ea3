// Handle, workspace layout and error reporting of libpfm.so.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "pfm_internal.cuh"

namespace pfm {

int set_error(pfm_handle* h, int status, const std::string& msg) {
  if (h) h->err = msg;
  return status;
}

int check_cuda(pfm_handle* h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PFM_OK;
  return set_error(h, PFM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int launch_check(pfm_handle* h, const char* what) { return check_cuda(h, cudaGetLastError(), what); }

int require_ws(pfm_handle* h) {
  if (!h->ws) return set_error(h, PFM_ERR_WORKSPACE, "no workspace bound (pfm_set_workspace)");
  if (h->ws_bytes < h->ws_need) return set_error(h, PFM_ERR_WORKSPACE, "workspace too small");
  return PFM_OK;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// ---- GraphCursor ------------------------------------------------------------------------------
cudaStream_t GraphCursor::seg() {
  if (open) return cs;
  cudaGraph_t target = G;
  const cudaGraphNode_t* d = deps;
  size_t nd = ndeps;
  if (rc) {  // keep later launches out of the stream: capture them into a graph that is dropped
    if (!junk && cudaGraphCreate(&junk, 0) != cudaSuccess) junk = nullptr;
    target = junk;
    d = nullptr;
    nd = 0;
  }
  const cudaError_t e = target ? cudaStreamBeginCaptureToGraph(cs, target, d, nullptr, nd, cudaStreamCaptureModeThreadLocal)
                               : cudaErrorInvalidValue;
  if (e != cudaSuccess) {
    if (!rc) rc = check_cuda(h, e, "begin graph segment");
    return cs;
  }
  open = true;
  return cs;
}

void GraphCursor::close() {
  if (!open) return;
  cudaStreamCaptureStatus cst;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* d = nullptr;
  size_t nd = 0;
  const cudaError_t e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &g, &d, nullptr, &nd);
  if (e == cudaSuccess && !junk && !rc) {
    if (nd > sizeof(deps) / sizeof(deps[0])) {
      rc = set_error(h, PFM_ERR_ARG, "graph segment ends in too many nodes");
    } else {
      for (size_t i = 0; i < nd; ++i) deps[i] = d[i];
      ndeps = nd;
    }
  }
  cudaGraph_t out = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(cs, &out);
  open = false;
  if (junk) {
    cudaGraphDestroy(junk);
    junk = nullptr;
  }
  if (!rc && e != cudaSuccess) rc = check_cuda(h, e, "graph segment info");
  if (!rc && e2 != cudaSuccess) rc = check_cuda(h, e2, "end graph segment");
}

cudaGraph_t GraphCursor::add_conditional(cudaGraphConditionalHandle cond, cudaGraphConditionalNodeType type) {
  close();
  if (rc) return nullptr;
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = type;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  rc = check_cuda(h, cudaGraphAddNode(&node, G, ndeps ? deps : nullptr, nullptr, ndeps, &cp), "conditional node");
  if (rc) return nullptr;
  deps[0] = node;
  ndeps = 1;
  return cp.conditional.phGraph_out[0];
}

int GraphCursor::begin_body(cudaGraph_t body) {
  return check_cuda(h, cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                    "begin body capture");
}

int GraphCursor::end_body() {
  cudaGraph_t b = nullptr;
  return check_cuda(h, cudaStreamEndCapture(cs, &b), "end body capture");
}

}  // namespace pfm

using namespace pfm;

extern "C" {

const char* pfm_status_string(int s) {
  switch (s) {
    case PFM_OK: return "ok";
    case PFM_ERR_NULL: return "null pointer";
    case PFM_ERR_SHAPE: return "shape mismatch";
    case PFM_ERR_WORKSPACE: return "workspace missing or too small";
    case PFM_ERR_NOT_CONVERGED: return "MGPCG did not converge";
    case PFM_ERR_NONFINITE: return "non-finite value";
    case PFM_ERR_CUDA: return "CUDA error";
    case PFM_ERR_ARG: return "invalid argument";
    default: return "unknown status";
  }
}

const char* pfm_last_error(const pfm_handle* h) { return h ? h->err.c_str() : "null handle"; }

int pfm_create(const pfm_config* cfg, pfm_handle** out) {
  if (!cfg || !out) return PFM_ERR_NULL;
  *out = nullptr;
  if (cfg->dim != 2 && cfg->dim != 3) return PFM_ERR_ARG;
  const int D = cfg->dim;
  for (int d = 0; d < D; ++d)
    if (cfg->res[d] < 4 || cfg->res[d] > (1 << 14)) return PFM_ERR_SHAPE;
  if (!(cfg->dx > 0.0)) return PFM_ERR_ARG;
  if (cfg->particles < 0) return PFM_ERR_ARG;
  pfm_handle* h = new (std::nothrow) pfm_handle();
  if (!h) return PFM_ERR_ARG;
  h->cfg = *cfg;
  if (D == 2) h->cfg.res[2] = 1;
  h->P = cfg->particles;
  MacGeom& g = h->geom;
  g.dim = D;
  for (int a = 0; a < 3; ++a) g.N[a] = (a < D) ? h->cfg.res[a] : 1;
  for (int c = 0; c < 3; ++c)
    for (int a = 0; a < 3; ++a) {
      g.n[c][a] = g.N[a] + ((a == c && c < D) ? 1 : 0);
      // u_dim - 2 - eps formed in double, rounded to f32 (3D/taichi_utils.py:282-284)
      g.hi[c][a] = (float)((double)g.n[c][a] - 2.0 - 1e-6);
    }
  g.dx = (float)cfg->dx;
  g.inv_dx = (float)(1.0 / cfg->dx);
  h->cells = (int64_t)g.N[0] * g.N[1] * g.N[2];
  // grid kernels index cells and faces with 32-bit integers
  for (int c = 0; c < D; ++c)
    if ((int64_t)g.n[c][0] * g.n[c][1] * g.n[c][2] >= (int64_t(1) << 31)) {
      delete h;
      return PFM_ERR_SHAPE;
    }
  for (int a = 0; a < 3; ++a) {
    g.dN[a] = make_div32((unsigned)g.N[a]);
    for (int c = 0; c < 3; ++c) g.dn[c][a] = make_div32((unsigned)g.n[c][a]);
  }

  // MGPCG hierarchy (3D/mgpcg.py:28): int(log2(min N)) - base_level + 1 levels
  int mn = g.N[0];
  for (int d = 1; d < D; ++d) mn = mn < g.N[d] ? mn : g.N[d];
  int L = (int)std::log2((double)mn) - cfg->base_level + 1;
  if (cfg->mg_levels > 0) L = cfg->mg_levels;
  if (L < 1 || L > kMaxLevels) {
    delete h;
    return PFM_ERR_ARG;
  }
  h->L = L;
  for (int l = 0; l < L; ++l) {
    int64_t cnt = 1;
    for (int a = 0; a < 3; ++a) {
      h->lv[l].n[a] = (a < D) ? (g.N[a] >> l) : 1;
      if (h->lv[l].n[a] < 1) {
        delete h;
        return PFM_ERR_SHAPE;
      }
      cnt *= h->lv[l].n[a];
    }
    h->lv[l].count = cnt;
  }
  if (h->cfg.pre_post_smoothing <= 0) h->cfg.pre_post_smoothing = 2;
  if (h->cfg.bottom_smoothing <= 0) h->cfg.bottom_smoothing = 50;

  // workspace layout
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  const size_t P = (size_t)h->P, C = (size_t)h->cells;
  h->o_key = take(P * 4);
  h->o_slot = take(P * 4);
  h->o_order = take(P * 4);
  h->o_count = take(C * 4);
  h->o_start = take((C + 1) * 4);
  size_t per_block = (size_t)kScanItems * kScanThreads;
  h->o_blocksums = take(((C + per_block - 1) / per_block + 1) * 4);
  // P2G records: pos4 + 3 impulse families (3D velocity), pos4 + 4 smoke channels (P2G_smoke)
  h->o_payload = take(P * 16 * (D == 3 ? 5 : 3));
  for (int l = 0; l < L; ++l) {
    h->o_r[l] = take((size_t)h->lv[l].count * 4);
    h->o_z[l] = take((size_t)h->lv[l].count * 4);
  }
  h->o_x = take(C * 4);
  h->o_p = take(C * 4);
  h->o_Ap = take(C * 4);
  h->o_b = take(C * 4);  // recentred right-hand side (warm start, true residual, tol_mode 2)
  h->o_partials = take(2 * kReduceBlocks * sizeof(double));  // two reductions in one pass (grid_sum2)
  h->o_state = take(sizeof(SolveState));
  h->o_maxpart = take(kReduceBlocks * sizeof(float) + 256);
  h->o_step = take(sizeof(StepCtl));
  h->o_x64 = take(C * 8);  // FP64 x of the residual-replacement solve
  h->o_hist = take(4 * C * 4);  // per pressure buffer: its last two solutions
  h->o_hist_flag = take(2 * sizeof(int));
  h->hist_ptr[0] = h->hist_ptr[1] = nullptr;

  h->ws_need = off;
  h->p2g2_column = 8;
  h->tail_cells = 4096;
  h->smooth_tma = 0;
  h->cube_kernels = 1;
  h->mid_centre = 1;
  if (cudaHostAlloc((void**)&h->h_state, sizeof(SolveState), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return PFM_ERR_CUDA;
  }
  std::memset(h->h_state, 0, sizeof(SolveState));
  *out = h;
  return PFM_OK;
}

int pfm_destroy(pfm_handle* h) {
  if (!h) return PFM_ERR_NULL;
  if (h->g_setup) cudaGraphExecDestroy(h->g_setup);
  if (h->g_loop) cudaGraphExecDestroy(h->g_loop);
  if (h->g_step) cudaGraphExecDestroy(h->g_step);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  if (h->h_state) cudaFreeHost(h->h_state);
  delete h;
  return PFM_OK;
}

int pfm_workspace_size(const pfm_handle* h, size_t* bytes) {
  if (!h || !bytes) return PFM_ERR_NULL;
  *bytes = h->ws_need;
  return PFM_OK;
}

int pfm_set_workspace(pfm_handle* h, void* dptr, size_t bytes) {
  if (!h) return PFM_ERR_NULL;
  if (!dptr) return set_error(h, PFM_ERR_NULL, "workspace pointer is NULL");
  if (((uintptr_t)dptr) & 255) return set_error(h, PFM_ERR_ARG, "workspace must be 256-byte aligned");
  if (bytes < h->ws_need) return set_error(h, PFM_ERR_WORKSPACE, "workspace smaller than pfm_workspace_size");
  if (h->ws != (char*)dptr) {  // a new workspace: the captured graphs and the step clock refer to the old one
    if (h->g_step) cudaGraphExecDestroy(h->g_step);
    if (h->g_setup) cudaGraphExecDestroy(h->g_setup);
    if (h->g_loop) cudaGraphExecDestroy(h->g_loop);
    h->g_step = h->g_setup = h->g_loop = nullptr;
    h->g_valid = 0;
    h->step_key.clear();
    h->step_clock_init = 0;
  }
  h->ws = (char*)dptr;
  h->ws_bytes = bytes;
  h->rec_valid = 0;
  // no pressure history yet in this workspace (warm_start 2)
  h->hist_ptr[0] = h->hist_ptr[1] = nullptr;
  const cudaError_t e = cudaMemset(ws_ptr<int>(h, h->o_hist_flag), 0, 2 * sizeof(int));
  if (e != cudaSuccess) return check_cuda(h, e, "pressure history flags");
  return PFM_OK;
}

int pfm_launch_count(const pfm_handle* h, uint64_t* launches) {
  if (!h || !launches) return PFM_ERR_NULL;
  *launches = h->launches;
  return PFM_OK;
}

int pfm_set_tuning(pfm_handle* h, int key, int value) {
  if (!h) return PFM_ERR_NULL;
  int rc = PFM_OK;
  if (key == PFM_TUNE_P2G2_COLUMN) {
    if (value < 1 || value > 64) return set_error(h, PFM_ERR_ARG, "P2G column length must be 1..64");
    h->p2g2_column = value;
  } else if (key == PFM_TUNE_MG_TAIL_CELLS) {
    rc = set_tail_cells(h, value);
  } else if (key == PFM_TUNE_SMOOTH_TMA) {
    if (value != 0 && value != 1) return set_error(h, PFM_ERR_ARG, "smoother staging must be 0 or 1");
    h->smooth_tma = value;
  } else if (key == PFM_TUNE_CUBE_KERNELS) {
    if (value != 0 && value != 1) return set_error(h, PFM_ERR_ARG, "cube kernels must be 0 or 1");
    h->cube_kernels = value;
  } else if (key == PFM_TUNE_MIDPOINT_CENTRE) {
    if (value != 0 && value != 1) return set_error(h, PFM_ERR_ARG, "midpoint face-centre form must be 0 or 1");
    h->mid_centre = value;
  } else {
    return set_error(h, PFM_ERR_ARG, "unknown tuning key");
  }
  if (rc) return rc;
  // captured graphs bake the old value in
  if (h->g_setup) cudaGraphExecDestroy(h->g_setup);
  if (h->g_loop) cudaGraphExecDestroy(h->g_loop);
  if (h->g_step) cudaGraphExecDestroy(h->g_step);
  h->g_setup = h->g_loop = h->g_step = nullptr;
  h->g_valid = 0;
  h->step_key.clear();
  return PFM_OK;
}

int pfm_get_tuning(const pfm_handle* h, int key, int* value) {
  if (!h || !value) return PFM_ERR_NULL;
  if (key == PFM_TUNE_P2G2_COLUMN) *value = h->p2g2_column;
  else if (key == PFM_TUNE_MG_TAIL_CELLS) *value = h->tail_cells;
  else if (key == PFM_TUNE_SMOOTH_TMA) *value = h->smooth_tma;
  else if (key == PFM_TUNE_CUBE_KERNELS) *value = h->cube_kernels;
  else if (key == PFM_TUNE_MIDPOINT_CENTRE) *value = h->mid_centre;
  else return PFM_ERR_ARG;
  return PFM_OK;
}

int pfm_mg_levels(const pfm_handle* h, int* levels) {
  if (!h || !levels) return PFM_ERR_NULL;
  *levels = h->L;
  return PFM_OK;
}

}  // extern "C"
