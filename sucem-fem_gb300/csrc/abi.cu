// C-ABI of libsucem_gb300: space construction, upload and assembly.
// Declarations and the reference interfaces they replace: include/sucem_gb300.h.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/sucem_gb300.h"
#include "device.h"
#include "n1curl_tables.h"
#include "space.h"
#include "handle.h"

namespace sucem {
void boundary_dual(const Space& hs, std::vector<double>& pt);
const double* n1curl_table_hi(int order, int which);
thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};
void count_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

int fail(const std::string& msg, int code) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  return fail(std::string(where) + ": " + cudaGetErrorString(e), SUCEM_ERR_CUDA);
}

namespace {

template <typename T>
cudaError_t up(T** dst, const T* src, size_t count) {
  *dst = nullptr;
  if (count == 0) return cudaSuccess;
  cudaError_t e = cudaMalloc((void**)dst, count * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
}

template <int ND>
void flatten_tables(const double (&kc)[6][ND][ND], const double (&km)[6][ND][ND],
                    const double (&kf)[4][3][ND][ND], std::vector<double>& c,
                    std::vector<double>& m, std::vector<double>& f) {
  c.assign(&kc[0][0][0], &kc[0][0][0] + 6 * ND * ND);
  m.assign(&km[0][0][0], &km[0][0][0] + 6 * ND * ND);
  f.assign(&kf[0][0][0][0], &kf[0][0][0][0] + 4 * 3 * ND * ND);
}

}  // namespace

void free_device_space(DeviceSpace* d) {
  if (!d) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(d->device);
  void* ptrs[] = {d->cells,   d->xyz_hi,  d->xyz_lo,    d->xyz,           d->ext_mask,
                  d->ent_ptr, d->inc_cell, d->inc_rec,  d->indptr,        d->indices,
                  d->cell_dofs, d->boundary_dofs, d->kc_f, d->km_f, d->kt_f,
                  d->kc_d,    d->km_d,    d->kt_d, d->bidx, d->g_f, d->g_d, d->g2_f, d->h2_f, d->kt_lo_f, d->h_f, d->h_d,
                  d->kab_f, d->kab_d, d->ext_facets, d->ntff_pts, d->bdof_pt,
                  d->bin_ptr, d->bin_cells, d->entry_ptr, d->entry_src, d->entry_perm, d->task_ent, d->task_meta,
                  d->step_words};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& kv : d->task_blocks)
    if (kv.second.first) cudaFree(kv.second.first);
  cudaSetDevice(prev);
  delete d;
}

std::string upload_space(Space& s, int device) {
  if (s.dev) {
    if (s.dev->device == device) return "";
    free_device_space(s.dev);
    s.dev = nullptr;
  }
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return std::string("cudaSetDevice: ") + cudaGetErrorString(e);
  DeviceSpace* d = new DeviceSpace();
  d->device = device;
  d->nt = s.nt;
  d->nv = s.nv;
  d->n = s.n;
  d->nnz = s.nnz;
  d->n_ent = s.n_ent;
  d->ninc = (int64_t)s.inc_cell.size();
  d->order = s.order;
  d->nd = s.ndof_cell;
  d->dpe = s.dofs_per_entity;
  d->rec_bytes = s.rec_bytes;
  d->max_row = s.max_row;
  std::vector<float4> hi(s.nv), lo(s.nv);
  for (int64_t v = 0; v < s.nv; ++v) {
    float h[3], l[3];
    for (int r = 0; r < 3; ++r) {
      double x = s.coords[v * 3 + r];
      h[r] = (float)x;
      l[r] = (float)(x - (double)h[r]);
    }
    hi[v] = make_float4(h[0], h[1], h[2], 0.f);
    lo[v] = make_float4(l[0], l[1], l[2], 0.f);
  }
  std::vector<int32_t> indptr32(s.n + 1);
  for (int64_t r = 0; r <= s.n; ++r) indptr32[r] = (int32_t)s.indptr[r];
  std::vector<double> kc, km, kf;
  if (s.order == 1) {
    flatten_tables<6>(KC1, KM1, KT1, kc, km, kf);
  } else if (s.order == 2) {
    flatten_tables<20>(KC2, KM2, KT2, kc, km, kf);
  } else {
    const size_t nn = (size_t)s.ndof_cell * s.ndof_cell;
    const double* tc = n1curl_table_hi(s.order, 0);
    const double* tm = n1curl_table_hi(s.order, 1);
    const double* tf = n1curl_table_hi(s.order, 2);
    if (!tc || !tm || !tf) {
      delete d;
      return "no reference tables for this order";
    }
    kc.assign(tc, tc + 6 * nn);
    km.assign(tm, tm + 6 * nn);
    kf.assign(tf, tf + 12 * nn);
  }
  std::vector<float> kcf(kc.begin(), kc.end()), kmf(km.begin(), km.end()),
      kff(kf.begin(), kf.end());
  const int nd = s.ndof_cell;
  std::vector<double> kab((size_t)nd * nd * 12);
  for (int a = 0; a < nd; ++a)
    for (int b = 0; b < nd; ++b)
      for (int m = 0; m < 6; ++m) {
        kab[((size_t)a * nd + b) * 12 + m] = kc[((size_t)m * nd + a) * nd + b];
        kab[((size_t)a * nd + b) * 12 + 6 + m] = km[((size_t)m * nd + a) * nd + b];
      }
  std::vector<float> kabf(kab.begin(), kab.end());
  std::vector<int32_t> bidx(s.nt);
  int64_t nb = 0;
  for (int64_t c = 0; c < s.nt; ++c) bidx[c] = s.ext_mask[c] ? (int32_t)nb++ : -1;
#define UP(field, src, cnt)                                                            \
  do {                                                                                 \
    e = up(&d->field, src, cnt);                                                       \
    if (e != cudaSuccess) {                                                            \
      std::string m = std::string("upload " #field ": ") + cudaGetErrorString(e);     \
      free_device_space(d);                                                            \
      return m;                                                                        \
    }                                                                                  \
  } while (0)
  UP(cells, reinterpret_cast<const int4*>(s.cells.data()), (size_t)s.nt);
  UP(xyz_hi, hi.data(), (size_t)s.nv);
  UP(xyz_lo, lo.data(), (size_t)s.nv);
  UP(xyz, s.coords.data(), (size_t)s.nv * 3);
  UP(ext_mask, s.ext_mask.data(), (size_t)s.nt);
  UP(indptr, indptr32.data(), indptr32.size());
  UP(indices, s.indices.data(), s.indices.size());
  UP(cell_dofs, s.cell_dofs.data(), s.cell_dofs.size());
  UP(boundary_dofs, s.boundary_dofs.data(), s.boundary_dofs.size());
  UP(kc_f, kcf.data(), kcf.size());
  UP(km_f, kmf.data(), kmf.size());
  UP(kt_f, kff.data(), kff.size());
  std::vector<float> kfl(kf.size());
  for (size_t i = 0; i < kf.size(); ++i) kfl[i] = (float)(kf[i] - (double)kff[i]);
  UP(kt_lo_f, kfl.data(), kfl.size());
  UP(kc_d, kc.data(), kc.size());
  UP(km_d, km.data(), km.size());
  UP(kt_d, kf.data(), kf.size());
  UP(kab_f, kabf.data(), kabf.size());
  UP(kab_d, kab.data(), kab.size());
  UP(bidx, bidx.data(), bidx.size());
  UP(entry_ptr, s.entry_ptr.data(), s.entry_ptr.size());
  UP(entry_src, s.entry_src.data(), s.entry_src.size());
  UP(entry_perm, s.entry_perm.data(), s.entry_perm.size());
  UP(task_ent, s.task_ent.data(), s.task_ent.size());
  UP(task_meta, reinterpret_cast<const int4*>(s.task_meta.data()), s.task_meta.size() / 4);
  UP(step_words, s.step_words.data(), s.step_words.size());
  d->task_P.resize(s.n_tasks);
  for (int64_t t = 0; t < s.n_tasks; ++t) d->task_P[t] = (uint16_t)((s.task_meta[t * 4 + 3] >> 8) & 0xffff);
  d->n_tasks = s.n_tasks;
  d->n_tasks_interior = s.n_tasks_interior;
  d->slot_planes = s.slot_planes;
  d->nb = nb;
#undef UP
  d->n_boundary = (int64_t)s.boundary_dofs.size();
  s.dev = d;
  return "";
}

}  // namespace sucem

using sucem::fail;
using sucem::cuda_fail;


extern "C" {

int sucem_version(void) { return SUCEM_ABI_VERSION; }

const char* sucem_last_error(void) { return sucem::g_last_error.c_str(); }

long long sucem_launch_count(void) { return sucem::g_launches.load(); }

int sucem_space_create(const double* coords, int64_t nv, const int64_t* cells, int64_t nt,
                       int order, sucem_space** out) {
  if (!coords || !cells || !out) return fail("null argument", SUCEM_ERR_ARG);
  *out = nullptr;
  sucem_space* h = new (std::nothrow) sucem_space();
  if (!h) return fail("out of host memory", SUCEM_ERR_MEMORY);
  std::string err;
  try {
    err = sucem::build_space(h->s, coords, nv, cells, nt, order);
  } catch (const std::bad_alloc&) {
    err = "out of host memory";
  }
  if (!err.empty()) {
    delete h;
    return fail(err, SUCEM_ERR_ARG);
  }
  *out = h;
  return SUCEM_OK;
}

void sucem_space_destroy(sucem_space* sp) {
  if (!sp) return;
  if (sp->s.dev) sucem::free_device_space(sp->s.dev);
  delete sp;
}

int sucem_space_sizes(const sucem_space* sp, int64_t* out) {
  if (!sp || !out) return fail("null argument", SUCEM_ERR_ARG);
  const sucem::Space& s = sp->s;
  out[0] = s.n;
  out[1] = s.nnz;
  out[2] = s.nv;
  out[3] = s.nt;
  out[4] = s.ne;
  out[5] = s.nf;
  out[6] = s.n_ext_facets;
  out[7] = (int64_t)s.boundary_dofs.size();
  out[8] = s.max_row;
  out[9] = (int64_t)s.inc_cell.size();
  return SUCEM_OK;
}

int sucem_space_schedule_sizes(const sucem_space* sp, int64_t* out) {
  if (!sp || !out) return fail("null argument", SUCEM_ERR_ARG);
  const sucem::Space& s = sp->s;
  out[0] = s.n_tasks;
  out[1] = s.n_tasks_interior;
  out[2] = s.slot_planes ? (int64_t)s.step_words.size() / ((1 + s.slot_planes) * 32) : 0;
  out[3] = s.slot_planes;
  return SUCEM_OK;
}

int sucem_space_copy(const sucem_space* sp, int what, void* dst) {
  if (!sp || !dst) return fail("null argument", SUCEM_ERR_ARG);
  const sucem::Space& s = sp->s;
  auto cp = [&](const void* src, size_t bytes) {
    if (bytes) std::memcpy(dst, src, bytes);
    return SUCEM_OK;
  };
  switch (what) {
    case SUCEM_COPY_INDPTR: return cp(s.indptr.data(), s.indptr.size() * 8);
    case SUCEM_COPY_INDICES: return cp(s.indices.data(), s.indices.size() * 4);
    case SUCEM_COPY_CELL_DOFS: return cp(s.cell_dofs.data(), s.cell_dofs.size() * 4);
    case SUCEM_COPY_BOUNDARY_DOFS: return cp(s.boundary_dofs.data(), s.boundary_dofs.size() * 4);
    case SUCEM_COPY_EDGES: return cp(s.edges.data(), s.edges.size() * 4);
    case SUCEM_COPY_FACES: return cp(s.faces.data(), s.faces.size() * 4);
    case SUCEM_COPY_CELLS: return cp(s.cells.data(), s.cells.size() * 4);
    case SUCEM_COPY_EXT_MASK: return cp(s.ext_mask.data(), s.ext_mask.size());
    case SUCEM_COPY_CELL_EDGES: return cp(s.cell_edges.data(), s.cell_edges.size() * 4);
    case SUCEM_COPY_CELL_FACES: return cp(s.cell_faces.data(), s.cell_faces.size() * 4);
    case SUCEM_COPY_DOF_XYZ: return cp(s.dof_xyz.data(), s.dof_xyz.size() * 8);
    case SUCEM_COPY_TASK_ENT: return cp(s.task_ent.data(), s.task_ent.size() * 4);
    case SUCEM_COPY_TASK_META: return cp(s.task_meta.data(), s.task_meta.size() * 4);
    case SUCEM_COPY_STEP_WORDS: return cp(s.step_words.data(), s.step_words.size() * 4);
    case SUCEM_COPY_ENTRY_PTR: return cp(s.entry_ptr.data(), s.entry_ptr.size() * 4);
    case SUCEM_COPY_ENTRY_SRC: return cp(s.entry_src.data(), s.entry_src.size() * 4);
    case SUCEM_COPY_ENTRY_PERM: return cp(s.entry_perm.data(), s.entry_perm.size() * 4);
    case SUCEM_COPY_BOUNDARY_DUAL: {
      if (s.order > 2) return fail("boundary dual functionals: basis orders 1 and 2 only", SUCEM_ERR_ARG);
      std::vector<double> pt;
      sucem::boundary_dual(s, pt);
      return cp(pt.data(), pt.size() * 8);
    }
    default: return fail("unknown copy selector", SUCEM_ERR_ARG);
  }
}

int sucem_space_upload(sucem_space* sp, int device) {
  if (!sp) return fail("null argument", SUCEM_ERR_ARG);
  std::string err = sucem::upload_space(sp->s, device);
  if (!err.empty()) return fail(err, SUCEM_ERR_CUDA);
  return SUCEM_OK;
}

int sucem_space_device_ptr(const sucem_space* sp, int what, void** out) {
  if (!sp || !out) return fail("null argument", SUCEM_ERR_ARG);
  const sucem::DeviceSpace* d = sp->s.dev;
  if (!d) return fail("space is not on a device (call sucem_space_upload)", SUCEM_ERR_STATE);
  switch (what) {
    case SUCEM_DEV_INDPTR: *out = d->indptr; break;
    case SUCEM_DEV_INDICES: *out = d->indices; break;
    case SUCEM_DEV_CELL_DOFS: *out = d->cell_dofs; break;
    case SUCEM_DEV_BOUNDARY_DOFS: *out = d->boundary_dofs; break;
    default: return fail("unknown device pointer selector", SUCEM_ERR_ARG);
  }
  return SUCEM_OK;
}

int sucem_assemble(const sucem_space* sp, int real_bytes, const void* eps_r,
                   const void* mu_r_inv, void* S, void* T, void* B, void* stream) {
  if (!sp) return fail("null space", SUCEM_ERR_ARG);
  if (real_bytes != 4 && real_bytes != 8) return fail("real_bytes must be 4 or 8", SUCEM_ERR_ARG);
  sucem::DeviceSpace* d = sp->s.dev;
  if (!d) return fail("space is not on a device (call sucem_space_upload)", SUCEM_ERR_STATE);
  if (!S && !T && !B) return SUCEM_OK;
  sucem::AssembleArgs a;
  a.real_bytes = real_bytes;
  a.mode = 0;
  a.eps_r = eps_r;
  a.mu_r_inv = mu_r_inv;
  a.S = S;
  a.T = T;
  a.B = B;
  cudaError_t e = sucem::launch_assemble(*d, a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_assemble");
  return SUCEM_OK;
}

int sucem_assemble_helmholtz(const sucem_space* sp, int real_bytes, const void* eps_r,
                             const void* mu_r_inv, double k0, void* A, void* stream) {
  if (!sp || !A) return fail("null argument", SUCEM_ERR_ARG);
  if (real_bytes != 4 && real_bytes != 8) return fail("real_bytes must be 4 or 8", SUCEM_ERR_ARG);
  sucem::DeviceSpace* d = sp->s.dev;
  if (!d) return fail("space is not on a device (call sucem_space_upload)", SUCEM_ERR_STATE);
  sucem::AssembleArgs a;
  a.real_bytes = real_bytes;
  a.mode = 1;
  a.eps_r = eps_r;
  a.mu_r_inv = mu_r_inv;
  a.A = A;
  a.k0 = k0;
  cudaError_t e = sucem::launch_assemble(*d, a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_assemble_helmholtz");
  return SUCEM_OK;
}

int sucem_assemble_host(const sucem_space* sp, int real_bytes, const void* eps_r_host,
                        const void* mu_r_inv_host, void* S_host, void* T_host, void* B_host) {
  if (!sp) return fail("null space", SUCEM_ERR_ARG);
  if (real_bytes != 4 && real_bytes != 8) return fail("real_bytes must be 4 or 8", SUCEM_ERR_ARG);
  sucem::DeviceSpace* d = sp->s.dev;
  if (!d) return fail("space is not on a device (call sucem_space_upload)", SUCEM_ERR_STATE);
  const size_t cbytes = (size_t)d->nt * real_bytes, vbytes = (size_t)d->nnz * real_bytes;
  void *de = nullptr, *dm = nullptr, *dS = nullptr, *dT = nullptr, *dB = nullptr;
  cudaError_t e = cudaSuccess;
  int rc = SUCEM_OK;
  auto take = [&](void** p, size_t b, bool need) {
    if (e == cudaSuccess && need) e = cudaMalloc(p, b);
  };
  take(&de, cbytes, eps_r_host != nullptr);
  take(&dm, cbytes, mu_r_inv_host != nullptr);
  take(&dS, vbytes, S_host != nullptr);
  take(&dT, vbytes, T_host != nullptr);
  take(&dB, vbytes, B_host != nullptr);
  if (e == cudaSuccess && de) e = cudaMemcpy(de, eps_r_host, cbytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && dm) e = cudaMemcpy(dm, mu_r_inv_host, cbytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    sucem::AssembleArgs a;
    a.real_bytes = real_bytes;
    a.eps_r = de;
    a.mu_r_inv = dm;
    a.S = dS;
    a.T = dT;
    a.B = dB;
    e = sucem::launch_assemble(*d, a, 0);
  }
  if (e == cudaSuccess && dS) e = cudaMemcpy(S_host, dS, vbytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && dT) e = cudaMemcpy(T_host, dT, vbytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && dB) e = cudaMemcpy(B_host, dB, vbytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = cuda_fail(e, "sucem_assemble_host");
  for (void* p : {de, dm, dS, dT, dB})
    if (p) cudaFree(p);
  return rc;
}

}  // extern "C"
