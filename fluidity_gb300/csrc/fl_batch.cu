// fl_batch.cu -- many scalar solves (fields on one mesh, or several meshes)
// assembled and solved together as CUDA graphs.
//
// Each member is one solve_field_equation_cg step (Advection_Diffusion_CG.F90:
// 127-174): element assembly, strong Dirichlet conditions, and an FP64 CG or
// GMRES(restart) + Jacobi solve with petsc_solve's ghost semantics.  The
// members are independent branches of one graph: the first graph runs every
// member's assembly, boundary conditions, solver set-up and a first chunk of
// iterations (CG: `chunk` iterations; GMRES: one restart cycle); then each
// member's graph of one more chunk is replayed, on the member's own stream,
// for the members whose device-side convergence flag is still clear.  The
// host reads one small array of flags between rounds, so a member that has
// converged costs nothing more (a graph of every member replayed as one
// would still launch its ~65-75 no-op kernels each round).  Results equal the
// members' individual solves bit for bit:
// each member has its own scratch and workspace, and every kernel sums in a
// fixed order.
#include <cstring>
#include <vector>

#include "fl_internal.cuh"
#include "fl_device.cuh"

namespace fl {

struct BatchMember {
  fl_mesh_t* m = nullptr;
  fl_advdif_params p{};
  fl_fields f{};
  int32_t nb = 0, base = 0;
  const int32_t* bc_nodes = nullptr;
  const double* bc_values = nullptr;
  fl_solver_opts o{};
  double* val = nullptr;
  double* rhs = nullptr;
  uint8_t* inactive = nullptr;
  double* x = nullptr;
  DevBuf<double> em;  // assembly scratch of this member
  CgPlan plan;
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;
};

}  // namespace fl

struct fl_batch_t {
  std::vector<fl::BatchMember*> mem;
  int chunk = 25;                       // iterations per replay of the iteration graph
  cudaGraphExec_t first = nullptr;      // assembly + set-up + first chunk
  std::vector<cudaGraphExec_t> iter;    // one chunk of iterations, per member
  fl::DevBuf<fl::KspState*> states;     // device array of member states
  fl::DevBuf<int> done;                 // gathered convergence flags
  int* h_done = nullptr;                // pinned host copy
  cudaStream_t s0 = nullptr;            // the batch's own stream (graphs are captured on it)
  cudaEvent_t fork = nullptr, join = nullptr;
  bool built = false;
};

using namespace fl;

static void destroy_graphs(fl_batch_t* b) {
  if (b->first) cudaGraphExecDestroy(b->first);
  for (cudaGraphExec_t e : b->iter)
    if (e) cudaGraphExecDestroy(e);
  b->first = nullptr;
  b->iter.clear();
  b->built = false;
}

extern "C" int fl_batch_create(fl_batch* out) {
  FL_CHECK_ARG(out, "null handle");
  fl_batch_t* b = new fl_batch_t();
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking) != cudaSuccess) {
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    delete b;
    set_error("stream/event creation failed");
    return FL_ERR_CUDA;
  }
  *out = b;
  return FL_OK;
}

extern "C" int fl_batch_destroy(fl_batch b) {
  if (!b) return FL_OK;
  cudaDeviceSynchronize();
  destroy_graphs(b);
  for (BatchMember* m : b->mem) {
    cg_release(m->plan);
    if (m->s) cudaStreamDestroy(m->s);
    if (m->ev) cudaEventDestroy(m->ev);
    delete m;
  }
  if (b->h_done) cudaFreeHost(b->h_done);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->s0) cudaStreamDestroy(b->s0);
  delete b;
  return FL_OK;
}

extern "C" int fl_batch_add(fl_batch b, fl_mesh mesh, const fl_advdif_params* params, const fl_fields* fields,
                            int32_t nb, const int32_t* bc_nodes, int32_t index_base, const double* bc_values,
                            const fl_solver_opts* opts, double* val, double* rhs, uint8_t* inactive, double* x) {
  FL_CHECK_ARG(b && mesh && params && fields && opts && val && rhs && inactive && x, "null argument");
  FL_CHECK_ARG(nb >= 0 && (nb == 0 || (bc_nodes && bc_values)), "boundary node list");
  FL_CHECK_ARG(index_base == 0 || index_base == 1, "index_base 0 or 1");
  FL_CHECK_ARG((opts->ksp_type == 0 || opts->ksp_type == 1) && opts->precision == 0,
               "batched members solve with FP64 CG or GMRES");
  BatchMember* m = new BatchMember();
  m->m = mesh;
  m->p = *params;
  m->f = *fields;
  m->nb = nb;
  m->bc_nodes = bc_nodes;
  m->base = index_base;
  m->bc_values = bc_values;
  m->o = *opts;
  m->val = val;
  m->rhs = rhs;
  m->inactive = inactive;
  m->x = x;
  if (cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&m->ev, cudaEventDisableTiming) != cudaSuccess) {
    delete m;
    set_error("stream/event creation failed");
    return FL_ERR_CUDA;
  }
  b->mem.push_back(m);
  destroy_graphs(b);
  return FL_OK;
}

// Enqueue one member's assembly, boundary conditions and solver set-up.
static int member_front(BatchMember* m, cudaStream_t s) {
  // the per-mesh assembly timer is not part of a captured graph
  const bool timing = m->m->timing;
  m->m->timing = false;
  const int st = assemble(m->m, &m->p, &m->f, m->val, m->rhs, s, m->em.p);
  m->m->timing = timing;
  FL_TRY(st);
  FL_TRY_CUDA(cudaMemsetAsync(m->inactive, 0, (size_t)m->m->N, s));
  FL_TRY(dirichlet_launch(m->m, m->nb, m->bc_nodes, m->base, m->bc_values, m->f.t, m->p.dt, m->rhs, m->inactive, s));
  cg_setup_launch(m->plan, s);
  return FL_OK;
}

// Capture `body` for every member on its own branch of a graph rooted at s0.
template <class Body>
static int capture(fl_batch_t* b, cudaStream_t s0, cudaGraphExec_t* exec, Body body) {
  cudaGraph_t g = nullptr;
  FL_TRY_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  int st = FL_OK;
  if (cudaEventRecord(b->fork, s0) != cudaSuccess) st = FL_ERR_CUDA;
  for (BatchMember* m : b->mem) {
    if (st != FL_OK) break;
    if (cudaStreamWaitEvent(m->s, b->fork, 0) != cudaSuccess) { st = FL_ERR_CUDA; break; }
    st = body(m);
    if (st == FL_OK && cudaEventRecord(m->ev, m->s) != cudaSuccess) st = FL_ERR_CUDA;
    if (st == FL_OK && cudaStreamWaitEvent(s0, m->ev, 0) != cudaSuccess) st = FL_ERR_CUDA;
  }
  gather_done(b->states.p, (int)b->mem.size(), b->done.p, s0);
  cudaError_t e = cudaStreamEndCapture(s0, &g);
  if (st != FL_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    set_error("graph capture failed: %s", cudaGetErrorString(e));
    return st != FL_OK ? st : FL_ERR_CUDA;
  }
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    set_error("graph instantiation failed: %s", cudaGetErrorString(e));
    return FL_ERR_CUDA;
  }
  return FL_OK;
}

static int build(fl_batch_t* b, cudaStream_t s0) {
  const int nm = (int)b->mem.size();
  FL_CHECK_ARG(nm > 0, "empty batch");
  // Preparation that may allocate or synchronise: scratch, workspaces, the
  // sliced layouts, the reference tables and kernel attributes (one ordinary
  // assembly per member configures them).
  std::vector<KspState*> hs(nm);
  for (int i = 0; i < nm; ++i) {
    BatchMember* m = b->mem[i];
    if (!m->m->tuned) FL_TRY(autotune_assembly(m->m, &m->p, &m->f, m->val, m->rhs, s0));
    FL_TRY(m->em.reserve(assembly_scratch_doubles(m->m, &m->p)));
    FL_TRY(cg_prepare(m->plan, m->m, &m->o, m->val, m->inactive, m->rhs, m->x, s0));
    FL_TRY(assemble(m->m, &m->p, &m->f, m->val, m->rhs, s0, m->em.p));
    hs[i] = cg_state(m->plan);
  }
  FL_TRY(b->states.reserve(nm));
  FL_TRY(b->done.reserve(nm));
  FL_TRY_CUDA(cudaMemcpyAsync(b->states.p, hs.data(), sizeof(KspState*) * nm, cudaMemcpyHostToDevice, s0));
  if (b->h_done) cudaFreeHost(b->h_done);
  FL_TRY_CUDA(cudaMallocHost(&b->h_done, sizeof(int) * nm));
  FL_TRY_CUDA(cudaStreamSynchronize(s0));
  const int chunk = b->chunk;
  auto steps = [&](BatchMember* m) { return m->o.ksp_type == 1 ? 1 : chunk; };
  FL_TRY(capture(b, s0, &b->first, [&](BatchMember* m) -> int {
    FL_TRY(member_front(m, m->s));
    for (int k = 0; k < steps(m); ++k) cg_iterate(m->plan, m->s);
    return FL_OK;
  }));
  b->iter.assign(nm, nullptr);
  for (int i = 0; i < nm; ++i) {
    BatchMember* m = b->mem[i];
    cudaGraph_t g = nullptr;
    FL_TRY_CUDA(cudaStreamBeginCapture(m->s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < steps(m); ++k) cg_iterate(m->plan, m->s);
    cudaError_t e = cudaStreamEndCapture(m->s, &g);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->iter[i], g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      set_error("graph capture failed: %s", cudaGetErrorString(e));
      return FL_ERR_CUDA;
    }
  }
  b->built = true;
  return FL_OK;
}

extern "C" int fl_batch_run(fl_batch b, void* stream, fl_solve_report* reports) {
  FL_CHECK_ARG(b && reports, "null argument");
  // the batch runs on its own stream (which can be captured), after the
  // caller's stream has reached this call and before it continues
  cudaStream_t caller = (cudaStream_t)stream;
  cudaStream_t s0 = b->s0;
  if (caller) {
    FL_TRY_CUDA(cudaEventRecord(b->join, caller));
    FL_TRY_CUDA(cudaStreamWaitEvent(s0, b->join, 0));
  }
  int st = FL_OK;
  do {
    if (!b->built && (st = build(b, s0)) != FL_OK) break;
    const int nm = (int)b->mem.size();
    // replays needed by the slowest member to reach its iteration limit
    int max_replays = 1;
    for (BatchMember* m : b->mem) {
      const int per = m->o.ksp_type == 1 ? m->plan.restart : b->chunk;
      const int r = (m->o.max_its + per - 1) / per + 1;
      max_replays = max_replays > r ? max_replays : r;
    }
    if (cudaGraphLaunch(b->first, s0) != cudaSuccess) { st = FL_ERR_CUDA; break; }
    for (int r = 0; r <= max_replays; ++r) {
      if (cudaMemcpyAsync(b->h_done, b->done.p, sizeof(int) * nm, cudaMemcpyDeviceToHost, s0) != cudaSuccess ||
          cudaStreamSynchronize(s0) != cudaSuccess) {
        st = FL_ERR_CUDA;
        break;
      }
      bool all = true;
      for (int i = 0; i < nm; ++i) all = all && b->h_done[i];
      if (all) break;
      // one more chunk of every member still running, each on its own stream
      if (cudaEventRecord(b->fork, s0) != cudaSuccess) { st = FL_ERR_CUDA; break; }
      for (int i = 0; i < nm && st == FL_OK; ++i) {
        if (b->h_done[i]) continue;
        BatchMember* m = b->mem[i];
        if (cudaStreamWaitEvent(m->s, b->fork, 0) != cudaSuccess || cudaGraphLaunch(b->iter[i], m->s) != cudaSuccess ||
            cudaEventRecord(m->ev, m->s) != cudaSuccess || cudaStreamWaitEvent(s0, m->ev, 0) != cudaSuccess)
          st = FL_ERR_CUDA;
      }
      if (st != FL_OK) break;
      gather_done(b->states.p, nm, b->done.p, s0);
    }
    if (st != FL_OK) break;
    for (BatchMember* m : b->mem) cg_finish_launch(m->plan, s0);
    for (int i = 0; i < nm && st == FL_OK; ++i) st = cg_report(b->mem[i]->plan, &reports[i], s0);
    if (st != FL_OK) break;
    for (BatchMember* m : b->mem)
      if ((st = check_err(m->m->err.p, s0, "batched assembly")) != FL_OK) break;
  } while (0);
  if (st == FL_ERR_CUDA && fl_last_error()[0] == 0) set_error("%s", cudaGetErrorString(cudaGetLastError()));
  if (caller && cudaEventRecord(b->join, s0) == cudaSuccess) cudaStreamWaitEvent(caller, b->join, 0);
  return st;
}

extern "C" int fl_batch_size(fl_batch b) { return b ? (int)b->mem.size() : 0; }

