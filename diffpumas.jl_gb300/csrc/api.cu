// api.cu -- context, error handling and physics-table handles of libdpgpu.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "internal.h"

namespace dp {
int fail(dp_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}
int cuda_fail(dp_ctx* ctx, cudaError_t e, const char* where) {
  return fail(ctx, DP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
void* scratch(dp_ctx* ctx, size_t bytes, int slot) {
  if (slot < 0 || slot > 3) return nullptr;
  void*& p = ctx->slot[slot];
  size_t& have = ctx->slot_bytes[slot];
  if (bytes <= have && p) return p;
  if (p) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(p);
  }
  p = nullptr;
  have = 0;
  size_t want = bytes + bytes / 4 + 256;
  if (cudaMalloc(&p, want) != cudaSuccess) return nullptr;
  have = want;
  return p;
}
static cudaEvent_t take_event(dp_ctx* ctx) {
  cudaEvent_t e = nullptr;
  if (!ctx->spare.empty()) {
    e = ctx->spare.back();
    ctx->spare.pop_back();
  } else {
    cudaEventCreate(&e);
  }
  return e;
}
// Resolves recorded event pairs into ctx->ktime (synchronises on them).
static void resolve_timing(dp_ctx* ctx) {
  for (auto& p : ctx->pending) {
    cudaEventSynchronize(p.b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    bool found = false;
    for (auto& kv : ctx->ktime)
      if (kv.name == p.name) {
        kv.ms += ms;
        ++kv.n;
        found = true;
      }
    if (!found) ctx->ktime.push_back({p.name, double(ms), 1});
    ctx->spare.push_back(p.a);
    ctx->spare.push_back(p.b);
  }
  ctx->pending.clear();
}
void timed_begin(dp_ctx* ctx) {
  ++ctx->launches;
  if (!ctx->timing) return;
  if (ctx->pending.size() >= 4096) resolve_timing(ctx);
  ctx->ev0 = take_event(ctx);
  cudaEventRecord(ctx->ev0, ctx->stream);
}
void timed_end(dp_ctx* ctx, const char* name) {
  if (!ctx->timing || !ctx->ev0) return;
  cudaEvent_t b = take_event(ctx);
  cudaEventRecord(b, ctx->stream);
  ctx->pending.push_back({name, ctx->ev0, b});
  ctx->ev0 = nullptr;
}
}  // namespace dp

using dp::fail;

extern "C" {

int dp_version(void) { return DPGPU_VERSION; }

int dp_init(int device, dp_ctx** out) {
  if (!out) return DP_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return DP_ERR_CUDA;
  if (device < 0 || device >= n) return DP_ERR_ARG;
  dp_ctx* c = new (std::nothrow) dp_ctx;
  if (!c) return DP_ERR_ALLOC;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaMalloc(&c->d_flag, sizeof(int)) != cudaSuccess ||
      cudaMemset(c->d_flag, 0, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&c->d_work, sizeof(unsigned long long)) != cudaSuccess) {
    if (c->d_flag) cudaFree(c->d_flag);
    delete c;
    return DP_ERR_CUDA;
  }
  c->stream = c->own_stream;
  *out = c;
  return DP_OK;
}

int dp_destroy(dp_ctx* c) {
  if (!c) return DP_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (void* s : c->slot)
    if (s) cudaFree(s);
  if (c->d_flag) cudaFree(c->d_flag);
  if (c->d_work) cudaFree(c->d_work);
  if (c->nodes_dev) cudaFree(c->nodes_dev);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t e : c->spare) cudaEventDestroy(e);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  cudaGetLastError();  // a failed release must not surface at a later launch
  delete c;
  return DP_OK;
}

int dp_set_stream(dp_ctx* c, void* stream) {
  if (!c) return DP_ERR_ARG;
  cudaStreamSynchronize(c->stream);
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return DP_OK;
}

void* dp_get_stream(const dp_ctx* c) { return c ? static_cast<void*>(c->stream) : nullptr; }

int dp_set_timing(dp_ctx* c, int enable) {
  if (!c) return DP_ERR_ARG;
  dp::resolve_timing(c);
  c->timing = enable ? 1 : 0;
  c->ktime.clear();
  return DP_OK;
}

int dp_kernel_time(dp_ctx* c, const char* name, double* ms) {
  return dp_kernel_stats(c, name, ms, nullptr);
}

int dp_kernel_stats(dp_ctx* c, const char* name, double* ms, long long* launches) {
  if (!c || !name || !ms) return DP_ERR_ARG;
  dp::resolve_timing(c);
  *ms = 0.0;
  if (launches) *launches = 0;
  for (const auto& kv : c->ktime)
    if (kv.name == name) {
      *ms = kv.ms;
      if (launches) *launches = kv.n;
    }
  return DP_OK;
}

long long dp_launch_count(const dp_ctx* c) { return c ? c->launches : -1; }

long long dp_scratch_bytes(const dp_ctx* c) {
  if (!c) return -1;
  long long b = 0;
  for (size_t s : c->slot_bytes) b += (long long)s;
  return b;
}

int dp_set_blocking(dp_ctx* c, int blocking) {
  if (!c) return DP_ERR_ARG;
  c->blocking = blocking ? 1 : 0;
  return DP_OK;
}

int dp_set_debug_limits(dp_ctx* c, int step_cap, int event_cap, int wait_iters) {
  if (!c) return DP_ERR_ARG;
  c->dbg_step_cap = step_cap < 0 ? -1 : step_cap;
  c->dbg_event_cap = event_cap < 0 ? -1 : event_cap;
  c->dbg_wait = wait_iters < 0 ? -1 : wait_iters;
  return DP_OK;
}

int dp_sync(dp_ctx* c) {
  if (!c) return DP_ERR_ARG;
  int flag = 0;
  if (cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return dp::fail(c, DP_ERR_CUDA, "stream synchronisation failed");
  if (flag) {
    cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream);
    cudaStreamSynchronize(c->stream);
    return dp::fail(c, DP_ERR_STATE, flag == 2   ? "ray segment buffer overflow"
                                     : flag == 4 ? "a CSDA history reached the transport step cap"
                                                 : "a kernel wait exceeded its limit");
  }
  return DP_OK;
}

const char* dp_last_error(const dp_ctx* c) { return c ? c->err.c_str() : "null context"; }

static int finish_upload(dp_ctx* ctx, dp_physics* p, dp_physics** out) {
  // Uniform log grid detection (enables O(1) interval lookup).
  const double* lE = &p->host[size_t(DP_COL_LOGE) * p->n];
  double d = (lE[p->n - 1] - lE[0]) / double(p->n - 1);
  bool uni = p->n > 2;
  for (int i = 0; i < p->n && uni; ++i)
    if (std::fabs(lE[i] - (lE[0] + d * i)) > 1e-9 * std::fabs(d)) uni = false;
  // All materials must share the energy grid.
  for (int m = 1; m < p->n_mat; ++m)
    if (std::memcmp(&p->host[(size_t(m) * DP_NCOL + DP_COL_E) * p->n], &p->host[0],
                    sizeof(double) * p->n) != 0) {
      delete p;
      return fail(ctx, DP_ERR_ARG, "all materials must share one energy grid");
    }
  p->ld = dp::padded(p->n);
  std::vector<double> pad(size_t(p->n_mat) * DP_NCOL * p->ld, 0.0);
  for (int m = 0; m < p->n_mat; ++m)
    for (int c = 0; c < DP_NCOL; ++c)
      std::memcpy(&pad[(size_t(m) * DP_NCOL + c) * p->ld], &p->host[(size_t(m) * DP_NCOL + c) * p->n],
                  sizeof(double) * p->n);
  if (cudaSetDevice(ctx->device) != cudaSuccess ||
      cudaMalloc(&p->dev, pad.size() * sizeof(double)) != cudaSuccess) {
    delete p;
    return fail(ctx, DP_ERR_CUDA, "table allocation failed");
  }
  if (cudaMemcpy(p->dev, pad.data(), pad.size() * sizeof(double), cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    cudaFree(p->dev);
    delete p;
    return fail(ctx, DP_ERR_CUDA, "table upload failed");
  }
  // single-precision derived columns
  p->ld32 = dp::padded32(p->n);
  std::vector<float> t32(size_t(p->n_mat) * dp::kNC32 * p->ld32, 0.0f);
  for (int m = 0; m < p->n_mat; ++m) {
    const double* E = &p->host[(size_t(m) * DP_NCOL + DP_COL_E) * p->n];
    const double* L = &p->host[(size_t(m) * DP_NCOL + DP_COL_LOGE) * p->n];
    const double* R = &p->host[(size_t(m) * DP_NCOL + DP_COL_CSDA_R) * p->n];
    const double* S = &p->host[(size_t(m) * DP_NCOL + DP_COL_CSDA_S) * p->n];
    auto C = [&](int c) { return &t32[(size_t(m) * dp::kNC32 + c) * p->ld32]; };
    for (int i = 0; i < p->n; ++i) {
      float rh = float(R[i]);
      C(dp::C32_RH)[i] = rh;
      C(dp::C32_RL)[i] = float(R[i] - double(rh));
      C(dp::C32_S)[i] = float(S[i]);
      C(dp::C32_E)[i] = float(E[i]);
      C(dp::C32_LE)[i] = float(L[i]);
      if (i + 1 < p->n) {
        double dl = L[i + 1] - L[i];
        C(dp::C32_SLOPE)[i] = float(dl / (R[i + 1] - R[i]));
        C(dp::C32_DSDLE)[i] = float((S[i + 1] - S[i]) / dl);
        C(dp::C32_DLE)[i] = float(dl);
      }
    }
  }
  if (cudaMalloc(&p->dev32, t32.size() * sizeof(float)) != cudaSuccess ||
      cudaMemcpy(p->dev32, t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice) !=
          cudaSuccess) {
    cudaFree(p->dev);
    if (p->dev32) cudaFree(p->dev32);
    delete p;
    return fail(ctx, DP_ERR_CUDA, "table upload failed");
  }
  p->view.base = p->dev;
  p->view.n = p->n;
  p->view.ld = p->ld;
  p->view.n_mat = p->n_mat;
  p->view.uniform = uni ? 1 : 0;
  p->view.lE0 = lE[0];
  p->view.inv_dlE = 1.0 / d;
  p->ctx = ctx;
  p->device = ctx->device;
  *out = p;
  return DP_OK;
}

static bool to_host_material(const dp_material& m, dp::HostMaterial& h) {
  if (m.n_elements <= 0 || !m.elements) return false;
  h.name = m.name ? m.name : "";
  h.density = m.density;
  h.I = m.I;
  double tot = 0.0;
  for (int i = 0; i < m.n_elements; ++i) tot += m.elements[i].fraction;
  if (!(tot > 0.0)) return false;
  double zoa = 0.0;
  h.elements.clear();
  for (int i = 0; i < m.n_elements; ++i) {
    const dp_element& e = m.elements[i];
    double f = e.fraction / tot;
    h.elements.push_back({e.Z, e.A, e.I, f});
    zoa += e.Z / e.A * f;
  }
  h.ZoA = m.ZoA > 0.0 ? m.ZoA : zoa;
  return true;
}

int dp_physics_upload(dp_ctx* ctx, const dp_settings* st, int n_mat, int n, const double* cols,
                      const dp_material* recipes, dp_physics** out) {
  if (!ctx || !st || !cols || !out || n_mat <= 0 || n < 2) return fail(ctx, DP_ERR_ARG, "bad arguments");
  dp_physics* p = new dp_physics;
  p->settings = *st;
  p->n_mat = n_mat;
  p->n = n;
  p->host.assign(cols, cols + size_t(n_mat) * DP_NCOL * n);
  if (recipes) {
    p->recipes.resize(n_mat);
    for (int m = 0; m < n_mat; ++m)
      if (!to_host_material(recipes[m], p->recipes[m])) {
        delete p;
        return fail(ctx, DP_ERR_ARG, "invalid material recipe");
      }
    p->has_recipes = true;
  }
  return finish_upload(ctx, p, out);
}

int dp_physics_create(dp_ctx* ctx, const dp_settings* st, int n_mat, const dp_material* mats,
                      int n, double Kmin, double Kmax, dp_physics** out) {
  if (!ctx || !st || !mats || !out || n_mat <= 0 || n < 2 || !(Kmin > 0.0) || !(Kmax > Kmin))
    return fail(ctx, DP_ERR_ARG, "bad arguments");
  dp_physics* p = new dp_physics;
  p->settings = *st;
  p->n_mat = n_mat;
  p->n = n;
  p->host.assign(size_t(n_mat) * DP_NCOL * n, 0.0);
  p->recipes.resize(n_mat);
  for (int m = 0; m < n_mat; ++m) {
    if (!to_host_material(mats[m], p->recipes[m])) {
      delete p;
      return fail(ctx, DP_ERR_ARG, "invalid material recipe");
    }
    dp::build_empirical_table(p->recipes[m], *st, n, Kmin, Kmax,
                              &p->host[size_t(m) * DP_NCOL * n]);
  }
  p->has_recipes = true;
  return finish_upload(ctx, p, out);
}

int dp_tables_from_dedx(const dp_settings* st, int n_mat, const dp_material* mats,
                        const char* const* dedx_paths, int* n_energies, double* cols,
                        long cap) {
  if (!st || n_mat <= 0 || !mats || !dedx_paths || !n_energies) return DP_ERR_ARG;
  std::vector<dp::DedxTable> t(n_mat);
  std::string err;
  for (int m = 0; m < n_mat; ++m) {
    if (!dedx_paths[m] || !dp::load_dedx_table(dedx_paths[m], &t[m], &err)) return DP_ERR_ARG;
    if (t[m].K != t[0].K) return DP_ERR_ARG;  // one energy grid for every material
  }
  const int n = int(t[0].K.size());
  *n_energies = n;
  if (!cols) return DP_OK;
  if (cap < long(n_mat) * DP_NCOL * n) return DP_ERR_ARG;
  for (int m = 0; m < n_mat; ++m) {
    dp::HostMaterial h;
    if (!to_host_material(mats[m], h)) return DP_ERR_ARG;
    dp::build_dedx_table(h, t[m], *st, cols + size_t(m) * DP_NCOL * n);
  }
  return DP_OK;
}

int dp_physics_create_dedx(dp_ctx* ctx, const dp_settings* st, int n_mat,
                           const dp_material* mats, const char* const* dedx_paths,
                           dp_physics** out) {
  if (!ctx || !st || !mats || !dedx_paths || !out || n_mat <= 0)
    return fail(ctx, DP_ERR_ARG, "bad arguments");
  std::vector<dp::DedxTable> t(n_mat);
  std::string err;
  for (int m = 0; m < n_mat; ++m) {
    if (!dedx_paths[m]) return fail(ctx, DP_ERR_ARG, "missing dE/dx file path");
    if (!dp::load_dedx_table(dedx_paths[m], &t[m], &err)) return fail(ctx, DP_ERR_ARG, err);
    if (t[m].K != t[0].K)
      return fail(ctx, DP_ERR_ARG, "the dE/dx files do not share one energy grid");
  }
  dp_physics* p = new dp_physics;
  p->settings = *st;
  p->n_mat = n_mat;
  p->n = int(t[0].K.size());
  p->host.assign(size_t(n_mat) * DP_NCOL * p->n, 0.0);
  p->recipes.resize(n_mat);
  for (int m = 0; m < n_mat; ++m) {
    if (!to_host_material(mats[m], p->recipes[m])) {
      delete p;
      return fail(ctx, DP_ERR_ARG, "invalid material recipe");
    }
    dp::build_dedx_table(p->recipes[m], t[m], *st, &p->host[size_t(m) * DP_NCOL * p->n]);
    p->recipes[m].ZoA = t[m].ZoA;
  }
  p->has_recipes = true;
  return finish_upload(ctx, p, out);
}

// Portable table file (little-endian, the byte order of x86-64 and AArch64):
//   "DPGPUTAB" | u32 version (1) | u32 n_materials | u32 n_energies |
//   u32 has_recipes | f64 mass, ctau, cutoff, elastic_ratio |
//   per material (has_recipes): u32 name length, name bytes, f64 density,
//   I, ZoA, u32 n_elements, n_elements x f64 (Z, A, I, fraction) |
//   n_materials x DP_NCOL x n_energies f64 columns (dp_column order).
}  // extern "C"
namespace {
constexpr char kTabMagic[8] = {'D', 'P', 'G', 'P', 'U', 'T', 'A', 'B'};
struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};
template <class T>
bool put(FILE* f, const T& v) {
  return std::fwrite(&v, sizeof(T), 1, f) == 1;
}
template <class T>
bool get(FILE* f, T* v) {
  return std::fread(v, sizeof(T), 1, f) == 1;
}
}  // namespace
extern "C" {

int dp_physics_save(const dp_physics* p, const char* path) {
  if (!p || !path) return DP_ERR_ARG;
  FileCloser fc{std::fopen(path, "wb")};
  FILE* f = fc.f;
  if (!f) return DP_ERR_ARG;
  bool ok = std::fwrite(kTabMagic, 1, 8, f) == 8 && put(f, uint32_t(1)) &&
            put(f, uint32_t(p->n_mat)) && put(f, uint32_t(p->n)) &&
            put(f, uint32_t(p->has_recipes ? 1 : 0)) && put(f, p->settings.mass) &&
            put(f, p->settings.ctau) && put(f, p->settings.cutoff) &&
            put(f, p->settings.elastic_ratio);
  if (ok && p->has_recipes)
    for (const auto& r : p->recipes) {
      ok = ok && put(f, uint32_t(r.name.size())) &&
           std::fwrite(r.name.data(), 1, r.name.size(), f) == r.name.size() &&
           put(f, r.density) && put(f, r.I) && put(f, r.ZoA) &&
           put(f, uint32_t(r.elements.size()));
      for (const auto& e : r.elements)
        ok = ok && put(f, e.Z) && put(f, e.A) && put(f, e.I) && put(f, e.fraction);
    }
  ok = ok && std::fwrite(p->host.data(), sizeof(double), p->host.size(), f) == p->host.size();
  return ok ? DP_OK : DP_ERR_ARG;
}

int dp_physics_load(dp_ctx* ctx, const char* path, dp_physics** out) {
  if (!ctx || !path || !out) return fail(ctx, DP_ERR_ARG, "bad arguments");
  FileCloser fc{std::fopen(path, "rb")};
  FILE* f = fc.f;
  if (!f) return fail(ctx, DP_ERR_ARG, std::string("cannot open ") + path);
  char magic[8];
  uint32_t version = 0, n_mat = 0, n = 0, has = 0;
  dp_settings st{};
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kTabMagic, 8) != 0 ||
      !get(f, &version) || version != 1 || !get(f, &n_mat) || !get(f, &n) || !get(f, &has) ||
      !get(f, &st.mass) || !get(f, &st.ctau) || !get(f, &st.cutoff) ||
      !get(f, &st.elastic_ratio) || n_mat == 0 || n_mat > 4096 || n < 2 || n > (1u << 24))
    return fail(ctx, DP_ERR_ARG, "not a version-1 physics table file");
  dp_physics* p = new dp_physics;
  p->settings = st;
  p->n_mat = int(n_mat);
  p->n = int(n);
  bool ok = true;
  if (has) {
    p->recipes.resize(n_mat);
    for (auto& r : p->recipes) {
      uint32_t len = 0, ne = 0;
      ok = ok && get(f, &len) && len < (1u << 16);
      if (!ok) break;
      r.name.resize(len);
      ok = ok && std::fread(&r.name[0], 1, len, f) == len && get(f, &r.density) &&
           get(f, &r.I) && get(f, &r.ZoA) && get(f, &ne) && ne < 4096;
      for (uint32_t k = 0; ok && k < ne; ++k) {
        dp::HostElement e{};
        ok = get(f, &e.Z) && get(f, &e.A) && get(f, &e.I) && get(f, &e.fraction);
        r.elements.push_back(e);
      }
    }
    p->has_recipes = ok;
  }
  p->host.resize(size_t(n_mat) * DP_NCOL * n);
  ok = ok && std::fread(p->host.data(), sizeof(double), p->host.size(), f) == p->host.size();
  if (!ok) {
    delete p;
    return fail(ctx, DP_ERR_ARG, "truncated physics table file");
  }
  return finish_upload(ctx, p, out);
}

int dp_physics_free(dp_physics* p) {
  if (!p) return DP_ERR_ARG;
  if (p->dev) {
    // the device saved at creation: the context may already be destroyed
    cudaSetDevice(p->device);
    cudaFree(p->dev);
    cudaFree(p->dev32);
    cudaGetLastError();  // a failed release must not surface at a later launch
  }
  delete p;
  return DP_OK;
}

int dp_physics_info(const dp_physics* p, int* n_mat, int* n) {
  if (!p) return DP_ERR_ARG;
  if (n_mat) *n_mat = p->n_mat;
  if (n) *n = p->n;
  return DP_OK;
}

int dp_physics_column(const dp_physics* p, int mat, int col, double* out) {
  if (!p || !out || mat < 0 || mat >= p->n_mat || col < 0 || col >= DP_NCOL) return DP_ERR_ARG;
  std::memcpy(out, &p->host[(size_t(mat) * DP_NCOL + col) * p->n], sizeof(double) * p->n);
  return DP_OK;
}

int dp_physics_settings(const dp_physics* p, dp_settings* out) {
  if (!p || !out) return DP_ERR_ARG;
  *out = p->settings;
  return DP_OK;
}

int dp_physics_material_name(const dp_physics* p, int m, char* buf, int cap) {
  if (!p || !p->has_recipes || m < 0 || m >= p->n_mat || !buf) return -1;
  const std::string& s = p->recipes[m].name;
  if (int(s.size()) + 1 > cap) return -1;
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return int(s.size());
}

int dp_physics_material_index(const dp_physics* p, const char* name) {
  if (!p || !name || !p->has_recipes) return -1;
  for (int m = 0; m < p->n_mat; ++m)
    if (p->recipes[m].name == name) return m;
  return -1;
}

}  // extern "C"
