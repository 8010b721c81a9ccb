// C ABI of libthreepoint_gb300.so: context, inputs, table build and the
// batched entry points. Host code only; kernels live in tp_tables.cu,
// tp_map3.cu, tp_gamma.cu and tp_cov.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "tp_bispec.cuh"
#include "tp_internal.cuh"
#include "tp_kernels.cuh"
#include "tp_tables.cuh"
#include "tp_capi_internal.h"
#include "tp_cubature.cuh"

using namespace tp;

// ---------------------------------------------------------------------------
// status helpers
// ---------------------------------------------------------------------------
extern "C" const char* tp_status_string(int s) {
  switch (s) {
    case TP_OK: return "ok";
    case TP_ERR_ARG: return "invalid argument";
    case TP_ERR_IO: return "file missing or unreadable";
    case TP_ERR_FORMAT: return "file content not in the expected format";
    case TP_ERR_CUDA: return "CUDA runtime error";
    case TP_ERR_STATE: return "call out of order";
    case TP_ERR_CAPACITY: return "an adaptive integral hit its region or sweep cap";
    case TP_ERR_NOMEM: return "out of memory";
  }
  return "unknown status";
}

extern "C" const char* tp_version(void) { return "threepoint_gb300 0.1 (sm_103a)"; }

extern "C" const char* tp_last_error(const tp_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int tp_fail(tp_ctx* ctx, int st, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return st;
}

int tp_cuda(tp_ctx* ctx, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return TP_OK;
  return tp_fail(ctx, TP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// inputs
// ---------------------------------------------------------------------------
extern "C" int tp_convert_angle_to_rad(double value, const char* unit, double* out) {
  if (!unit || !out) return TP_ERR_ARG;
  double c;
  if (!strcmp(unit, "arcmin"))
    c = 2.9088820866e-4;
  else if (!strcmp(unit, "deg"))
    c = 0.017453;
  else if (!strcmp(unit, "rad"))
    c = 1;
  else
    return TP_ERR_ARG;
  *out = c * value;
  return TP_OK;
}

static bool read_name_value_lines(const char* path, std::vector<std::pair<std::string, std::string>>& kv) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream iss(line);
    std::string n, v;
    iss >> n >> v;
    if (n.empty()) continue;
    kv.emplace_back(n, v);
  }
  return true;
}

extern "C" int tp_cosmology_from_file(const char* path, tp_cosmology* out) {
  if (!path || !out) return TP_ERR_ARG;
  std::vector<std::pair<std::string, std::string>> kv;
  if (!read_name_value_lines(path, kv)) return TP_ERR_IO;
  tp_cosmology c;
  memset(&c, 0, sizeof(c));
  int seen = 0;
  for (auto& p : kv) {
    double v = atof(p.second.c_str());
    if (p.first == "h") c.h = v, seen |= 1;
    else if (p.first == "sigma_8") c.sigma8 = v, seen |= 2;
    else if (p.first == "Omega_b") c.omb = v, seen |= 4;
    else if (p.first == "n_s") c.ns = v, seen |= 8;
    else if (p.first == "w") c.w = v, seen |= 16;
    else if (p.first == "Omega_m") c.om = v, seen |= 32;
    else if (p.first == "z_max") c.zmax = v, seen |= 64;
    else return TP_ERR_FORMAT;  // the reference stops at an unknown key
  }
  if (seen != 127) return TP_ERR_FORMAT;
  c.ow = 1 - c.om;
  c.omc = c.om - c.omb;
  *out = c;
  return TP_OK;
}

extern "C" int tp_cov_params_from_file(const char* path, tp_cov_params* out) {
  if (!path || !out) return TP_ERR_ARG;
  std::vector<std::pair<std::string, std::string>> kv;
  if (!read_name_value_lines(path, kv)) return TP_ERR_IO;
  tp_cov_params c;
  memset(&c, 0, sizeof(c));
  std::string unit;
  for (auto& p : kv) {
    const char* v = p.second.c_str();
    if (p.first == "thetaMax") c.theta_max = atof(v);
    else if (p.first == "thetaMax_smaller") c.theta_max_smaller = atof(v);
    else if (p.first == "shapenoise_sigma") c.shapenoise_sigma = atof(v);
    else if (p.first == "galaxy_density") c.galaxy_density = atof(v);
    else if (p.first == "unit") unit = p.second;
    else if (p.first == "shapenoiseOnly") c.shapenoise_only = atoi(v) != 0;
    else if (p.first == "area") c.area = atof(v);
    else return TP_ERR_FORMAT;
  }
  // unit conversion as at the end of the reference constructor (cosmology.cu:162-169)
  double one;
  if (tp_convert_angle_to_rad(1.0, unit.c_str(), &one)) return TP_ERR_FORMAT;
  c.theta_max *= one;
  c.theta_max_smaller *= one;
  c.area = c.area * one * one;
  c.galaxy_density = c.galaxy_density / one / one;
  *out = c;
  return TP_OK;
}

extern "C" int tp_gamma_config_from_file(const char* path, tp_gamma_config* out) {
  if (!path || !out) return TP_ERR_ARG;
  std::vector<std::pair<std::string, std::string>> kv;
  if (!read_name_value_lines(path, kv)) return TP_ERR_IO;
  tp_gamma_config c;
  memset(&c, 0, sizeof(c));
  int seen = 0;
  for (auto& p : kv) {
    const double v = atof(p.second.c_str());
    if (p.first == "rmin") c.rmin = v, seen |= 1;
    else if (p.first == "rmax") c.rmax = v, seen |= 2;
    else if (p.first == "umin") c.umin = v, seen |= 4;
    else if (p.first == "umax") c.umax = v, seen |= 8;
    else if (p.first == "vmin") c.vmin = v, seen |= 16;
    else if (p.first == "vmax") c.vmax = v, seen |= 32;
    else if (p.first == "rsteps") c.rsteps = (int)std::round(v), seen |= 64;
    else if (p.first == "usteps") c.usteps = (int)std::round(v), seen |= 128;
    else if (p.first == "vsteps") c.vsteps = (int)std::round(v), seen |= 256;
    else return TP_ERR_FORMAT;
  }
  if (seen != 511) return TP_ERR_FORMAT;
  *out = c;
  return TP_OK;
}

extern "C" int tp_gamma_triangles(const tp_gamma_config* cfg, double* x, double* ruv) {
  if (!cfg || !x || cfg->rsteps < 1 || cfg->usteps < 1 || cfg->vsteps < 1 || !(cfg->rmin > 0) || !(cfg->rmax > 0))
    return TP_ERR_ARG;
  const double lrmin = log(cfg->rmin), lrmax = log(cfg->rmax);
  long t = 0;
  for (int i = 0; i < cfg->rsteps; i++) {
    const double r = exp(lrmin + (lrmax - lrmin) / cfg->rsteps * (i + 0.5));
    for (int j = 0; j < cfg->usteps; j++) {
      const double u = cfg->umin + (cfg->umax - cfg->umin) / cfg->usteps * (j + 0.5);
      for (int k = 0; k < cfg->vsteps; k++, t++) {
        const double v = cfg->vmin + (cfg->vmax - cfg->vmin) / cfg->vsteps * (k + 0.5);
        const double r2 = r * M_PI / 180. / 60.;  // Jarvis et al. (2004) binning
        const double r3 = r2 * u;
        x[3 * t] = v * r3 + r2;
        x[3 * t + 1] = r2;
        x[3 * t + 2] = r3;
        if (ruv) ruv[3 * t] = r, ruv[3 * t + 1] = u, ruv[3 * t + 2] = v;
      }
    }
  }
  return TP_OK;
}

extern "C" int tp_rebin_n_of_z(const double* zs, const double* ns, int nf, int n_bins, double zmax, double* nz_out) {
  if (!zs || !ns || !nz_out || nf < 2 || n_bins <= 0 || !(zmax > 0)) return TP_ERR_ARG;
  const double zmin_f = zs[0], zmax_f = zs[nf - 1];
  const double dz_f = (zmax_f - zmin_f) / (nf - 1);
  const double dz = zmax / n_bins;
  std::vector<double> nz;
  nz.reserve(n_bins);
  if (dz > dz_f) {
    // linear interpolation of the finer file grid (helpers.cu:44-63)
    for (int i = 0; i < n_bins; i++) {
      double z = i * dz;
      int ix = int((z - zmin_f) / dz_f);
      double dix = (z - zmin_f) / dz_f - ix;
      double v = 0;
      if (ix >= 0 && ix < nf - 1) v = ns[ix + 1] * dix + ns[ix] * (1 - dix);
      if (ix >= nf - 1) v = 0.0;
      nz.push_back(v);
    }
  } else {
    // bin averaging of the coarser file grid (helpers.cu:64-114)
    for (int i = 0; i < n_bins; i++) {
      double zl = i * dz, zu = (i + 1) * dz;
      int k = 0, l = 0;
      for (int j = 0; j < nf; j++) {
        if (zs[j] < zl) k = j;
        if (zs[j] < zu) l = j;
      }
      double v = 0;
      if (zu < zmin_f || k > nf) {
        v = 0.0;
      } else if (l - k <= 1) {
        if (k == l)
          v = ns[k];
        else if (l > nf)
          v = ns[k] * (zs[l] - zl) / dz;
        else if (zl < zmin_f)
          v = ns[l] * (zu - zs[l]) / dz;
        else
          v = ns[k] * (zs[l] - zl) / dz + ns[l] * (zu - zs[l]) / dz;
      }
      nz.push_back(v);
    }
  }
  double norm = std::accumulate(nz.begin(), nz.end(), 0.0);
  if (norm == 0) return TP_ERR_FORMAT;
  norm *= dz;
  for (int i = 0; i < n_bins; i++) nz_out[i] = nz[i] / norm;
  return TP_OK;
}

extern "C" int tp_read_n_of_z(const char* path, int n_bins, double zmax, double* nz_out) {
  if (!path || !nz_out || n_bins <= 0 || !(zmax > 0)) return TP_ERR_ARG;
  std::ifstream in(path);
  if (!in) return TP_ERR_IO;
  std::vector<double> zs, ns;
  std::string line;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream iss(line);
    double z, n;
    if (!(iss >> z >> n)) return TP_ERR_FORMAT;
    zs.push_back(z);
    ns.push_back(n);
  }
  if (zs.size() < 2) return TP_ERR_FORMAT;
  return tp_rebin_n_of_z(zs.data(), ns.data(), (int)zs.size(), n_bins, zmax, nz_out);
}

extern "C" int tp_read_thetas(const char* path, double* out, int cap, int* n_out) {
  if (!path || !n_out) return TP_ERR_ARG;
  std::ifstream in(path);
  if (!in) return TP_ERR_IO;
  std::string line;
  int n = 0;
  while (std::getline(in, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream iss(line);
    double t;
    if (!(iss >> t)) return TP_ERR_FORMAT;
    if (out && n < cap) out[n] = t;
    ++n;
  }
  *n_out = n;
  return TP_OK;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
template <typename T>
static cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}

void tp_ctx::free_cosmo() {
  cudaFree(d_cos);
  cudaFree(d_eh);
  cudaFree(d_tab);
  cudaFree(d_nz);
  cudaFree(d_ncoef64);
  cudaFree(d_ncoef32);
  cudaFree(d_fcoef32);
  cudaFree(d_hcoef);
  cudaFree(d_hcoef32);
  cudaFree(d_wscale64);
  cudaFree(d_wscale32);
  cudaFree(d_ck64);
  cudaFree(d_ck32);
  cudaFree(d_plt);
  cudaFree(d_ehg);
  cudaFree(d_halo);
  d_halo = nullptr;
  halo_ready.clear();
  d_cos = nullptr;
  d_eh = nullptr;
  d_tab = nullptr;
  d_nz = nullptr;
  d_ncoef64 = nullptr;
  d_ncoef32 = nullptr;
  d_fcoef32 = nullptr;
  d_hcoef = nullptr;
  d_hcoef32 = nullptr;
  d_wscale64 = d_wscale32 = nullptr;
  d_ck64 = nullptr;
  d_ck32 = nullptr;
  d_plt = nullptr;
  d_ehg = nullptr;
  n_cosmo = 0;
  cosmo_cap = 0;
  nz_cap = 0;
}

int tp_ctx::ensure_scratch(size_t bytes) {
  if (bytes <= scratch_bytes) return TP_OK;
  cudaFree(d_scratch);
  d_scratch = nullptr;
  scratch_bytes = 0;
  cudaError_t e = cudaMalloc((void**)&d_scratch, bytes);
  if (e != cudaSuccess) return tp_cuda(this, e, "scratch allocation");
  scratch_bytes = bytes;
  return TP_OK;
}

int tp_ctx::ensure_io(size_t bytes) {
  if (bytes <= io_bytes) return TP_OK;
  cudaFree(d_io);
  d_io = nullptr;
  io_bytes = 0;
  cudaError_t e = cudaMalloc((void**)&d_io, bytes);
  if (e != cudaSuccess) return tp_cuda(this, e, "io allocation");
  io_bytes = bytes;
  return TP_OK;
}

extern "C" int tp_ctx_create(int device, tp_ctx** out) {
  if (!out) return TP_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TP_ERR_CUDA;
  if (device < 0 || device >= ndev) return TP_ERR_ARG;
  tp_ctx* c = new tp_ctx();
  c->device = device;
  cudaGetLastError();  // a stale error left by other code in the process is not this context's
  if (cudaSetDevice(device) != cudaSuccess) {
    delete c;
    return TP_ERR_CUDA;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_counter, 64);
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_diag, 64);
  if (e == cudaSuccess) e = cudaMemset(c->d_diag, 0, 64);
  if (e != cudaSuccess) {
    delete c;
    return TP_ERR_CUDA;
  }
  upload_gauss_nodes();
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    delete c;
    return TP_ERR_CUDA;
  }
  *out = c;
  return TP_OK;
}

extern "C" int tp_ctx_destroy(tp_ctx* c) {
  if (!c) return TP_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->free_cosmo();
  cudaFree(c->d_scratch);
  cudaFree(c->d_io);
  cudaFree(c->d_counter);
  cudaFree(c->d_diag);
  cudaStreamDestroy(c->stream);
  delete c;
  return TP_OK;
}

extern "C" int tp_set_cosmologies(tp_ctx* ctx, const tp_cosmology* cosmo, int n, const double* nz, int nz_stride,
                                  const double* pk, double dk, double kmin, double kmax) {
  TpRange nvtx_range("tp_set_cosmologies: table build");
  if (!ctx || !cosmo || n <= 0 || !nz || (nz_stride != 0 && nz_stride != NZ)) return TP_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    const tp_cosmology& c = cosmo[i];
    bool ok = c.zmax > 0 && c.zmax < 1e3 && c.om > 0 && c.om <= 1 && c.h > 0 && c.sigma8 >= 0 && c.omb >= 0 &&
              c.omb < c.om && std::isfinite(c.ns) && std::isfinite(c.w) && std::isfinite(c.ow) &&
              std::isfinite(c.omc) && std::isfinite(c.h) && std::isfinite(c.sigma8);
    if (!ok) return tp_fail(ctx, TP_ERR_ARG, "cosmology " + std::to_string(i) + " is outside the supported domain");
  }
  if (pk && !(kmin > 0 && kmax > kmin && dk > 0)) return tp_fail(ctx, TP_ERR_ARG, "invalid P(k) binning");
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  std::vector<CosmoDev> hc(n);
  std::vector<EHConst> he(n);
  for (int i = 0; i < n; ++i) {
    CosmoDev& c = hc[i];
    const tp_cosmology& s = cosmo[i];
    c.h = s.h;
    c.sigma8 = s.sigma8;
    c.omb = s.omb;
    c.omc = s.omc;
    c.ns = s.ns;
    c.w = s.w;
    c.om = s.om;
    c.ow = s.ow;
    c.zmax = s.zmax;
    c.pk_given = pk != nullptr;
    c.dk = dk;
    c.kmin = kmin;
    c.kmax = kmax;
    c.sigma_eps = ctx->sigma_eps;
    c.ngal = ctx->ngal;
    c.constant_ps = ctx->constant_ps;
    he[i] = make_eh_const(c, 1.0);
  }
  cudaError_t e = cudaSuccess;
  size_t nzn = nz_stride ? (size_t)n * NZ : NZ;
  // device buffers are kept and reused while the batch fits their capacity
  if (n > ctx->cosmo_cap || nzn > ctx->nz_cap) {
    ctx->free_cosmo();
    int cap = std::max(n, ctx->cosmo_cap);
    if (e == cudaSuccess) e = dalloc(&ctx->d_cos, cap);
    if (e == cudaSuccess) e = dalloc(&ctx->d_eh, cap);
    if (e == cudaSuccess) e = dalloc(&ctx->d_tab, cap);
    if (e == cudaSuccess) e = dalloc(&ctx->d_nz, (size_t)cap * NZ);
    if (e == cudaSuccess) e = dalloc(&ctx->d_ncoef64, (size_t)cap * NCP * NNODE);
    if (e == cudaSuccess) e = dalloc(&ctx->d_ncoef32, (size_t)cap * NCP * NNODE);
    if (e == cudaSuccess) e = dalloc(&ctx->d_fcoef32, (size_t)cap * NCP * NNODE);
    if (e == cudaSuccess) e = dalloc(&ctx->d_hcoef, (size_t)cap * HC_COUNT * NNODE);
    if (e == cudaSuccess) e = dalloc(&ctx->d_hcoef32, (size_t)cap * HC_COUNT * NNODE);
    if (e == cudaSuccess) e = dalloc(&ctx->d_wscale64, cap);
    if (e == cudaSuccess) e = dalloc(&ctx->d_wscale32, cap);
    if (e == cudaSuccess) e = dalloc((CosmoK<double>**)&ctx->d_ck64, cap);
    if (e == cudaSuccess) e = dalloc((CosmoK<float>**)&ctx->d_ck32, cap);
    if (e == cudaSuccess) e = dalloc(&ctx->d_plt, (size_t)cap * PLT_N);
    if (e == cudaSuccess) e = dalloc(&ctx->d_ehg, (size_t)cap * EHG_N);
    if (e != cudaSuccess) {
      ctx->free_cosmo();
      return tp_cuda(ctx, e, "cosmology allocation");
    }
    ctx->cosmo_cap = cap;
    ctx->nz_cap = (size_t)cap * NZ;
  }
  ctx->n_cosmo = n;
  ctx->h_cos = hc;
  ctx->halo_ready.assign(ctx->cosmo_cap, 0);
  cudaStream_t s = ctx->stream;
  e = cudaMemcpyAsync(ctx->d_cos, hc.data(), sizeof(CosmoDev) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->d_eh, he.data(), sizeof(EHConst) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->d_nz, nz, sizeof(double) * nzn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && pk)
    for (int i = 0; i < n && e == cudaSuccess; ++i)
      e = cudaMemcpyAsync((char*)ctx->d_tab + (size_t)i * sizeof(TablesDev) + offsetof(TablesDev, pk), pk + (size_t)i * NK, sizeof(double) * NK, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = build_tables(ctx->d_cos, ctx->d_eh, ctx->d_nz, nz_stride, ctx->d_tab, ctx->d_ncoef64, ctx->d_ncoef32,
                     ctx->d_fcoef32, ctx->d_hcoef, ctx->d_hcoef32, ctx->d_wscale64, ctx->d_wscale32, (CosmoK<double>*)ctx->d_ck64,
                     (CosmoK<float>*)ctx->d_ck32, ctx->d_plt, ctx->d_ehg, n, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "table build");
  return TP_OK;
}

extern "C" int tp_set_shape_noise(tp_ctx* ctx, double sigma_eps, double n_gal, int constant_ps) {
  if (!ctx || !(n_gal > 0) || sigma_eps < 0) return TP_ERR_ARG;
  ctx->sigma_eps = sigma_eps;
  ctx->ngal = n_gal;
  ctx->constant_ps = constant_ps != 0;
  return TP_OK;
}

extern "C" int tp_set_rectangle_side(tp_ctx* ctx, double theta_max_smaller) {
  if (!ctx || !(theta_max_smaller > 0)) return TP_ERR_ARG;
  ctx->theta_max_smaller = theta_max_smaller;
  return TP_OK;
}

extern "C" int tp_get_tables(tp_ctx* ctx, int i, double* out) {
  if (!ctx || !out) return TP_ERR_ARG;
  if (i < 0 || i >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_STATE, "no such cosmology");
  cudaSetDevice(ctx->device);
  TablesDev* t = new TablesDev;
  cudaError_t e = cudaMemcpyAsync(t, ctx->d_tab + i, sizeof(TablesDev), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    delete t;
    return tp_cuda(ctx, e, "tables copy");
  }
  memcpy(out + 0 * NZ, t->f_K, sizeof(double) * NZ);
  memcpy(out + 1 * NZ, t->g, sizeof(double) * NZ);
  memcpy(out + 2 * NZ, t->D1, sizeof(double) * NZ);
  memcpy(out + 3 * NZ, t->r_sigma, sizeof(double) * NZ);
  memcpy(out + 4 * NZ, t->n_eff, sizeof(double) * NZ);
  memcpy(out + 5 * NZ, t->ncur, sizeof(double) * NZ);
  out[6 * NZ] = t->norm;
  delete t;
  return TP_OK;
}

// ---------------------------------------------------------------------------
// point evaluations
// ---------------------------------------------------------------------------
extern "C" int tp_bkappa_batch(tp_ctx* ctx, const int* cosmo_index, const double* ell, long n, int precision,
                               double* out) {
  TpRange nvtx_range("tp_bkappa_batch");
  if (!ctx || !ell || !out || n < 0) return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  if (ctx->n_cosmo == 0) return tp_fail(ctx, TP_ERR_STATE, "no cosmology set");
  if (n == 0) return TP_OK;
  if (cosmo_index)
    for (long i = 0; i < n; ++i)
      if (cosmo_index[i] < 0 || cosmo_index[i] >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_ARG, "bad cosmology index");
  cudaSetDevice(ctx->device);
  size_t b_ell = sizeof(double) * 3 * n, b_out = sizeof(double) * n, b_idx = cosmo_index ? sizeof(int) * n : 0;
  size_t off_out = (b_ell + 255) & ~size_t(255), off_idx = (off_out + b_out + 255) & ~size_t(255);
  int st = ctx->ensure_io(off_idx + b_idx + 256);
  if (st) return st;
  char* base = ctx->d_io;
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(base, ell, b_ell, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && cosmo_index) e = cudaMemcpyAsync(base + off_idx, cosmo_index, b_idx, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = launch_bkappa_points(precision, cosmo_index ? (int*)(base + off_idx) : nullptr, (double*)base, n,
                             precision == TP_FP64 ? (const void*)ctx->d_ncoef64 : (const void*)ctx->d_fcoef32,
                             precision == TP_FP64 ? ctx->d_wscale64 : ctx->d_wscale32,
                             precision == TP_FP64 ? ctx->d_ck64 : ctx->d_ck32, (double*)(base + off_out), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, base + off_out, b_out, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return tp_cuda(ctx, e, "bkappa");
}

extern "C" int tp_bkappa_nodes(tp_ctx* ctx, int cosmo_index, const double* ell, long n, int precision, double* term,
                               double* bispec) {
  TpRange nvtx_range("tp_bkappa_nodes");
  if (!ctx || !ell || !term || n < 0) return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  if (cosmo_index < 0 || cosmo_index >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_STATE, "no such cosmology");
  if (n == 0) return TP_OK;
  cudaSetDevice(ctx->device);
  const size_t b_ell = sizeof(double) * 3 * n, b_node = sizeof(double) * NNODE * n;
  const size_t o_t = (b_ell + 255) & ~size_t(255), o_b = o_t + ((b_node + 255) & ~size_t(255));
  int st = ctx->ensure_io(o_b + b_node + 256);
  if (st) return st;
  char* base = ctx->d_io;
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(base, ell, b_ell, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = launch_bkappa_nodes(precision, cosmo_index, (const double*)base, n,
                            precision == TP_FP64 ? (const void*)ctx->d_ncoef64 : (const void*)ctx->d_fcoef32,
                            precision == TP_FP64 ? ctx->d_wscale64 : ctx->d_wscale32,
                            precision == TP_FP64 ? ctx->d_ck64 : ctx->d_ck32, (double*)(base + o_t),
                            bispec ? (double*)(base + o_b) : nullptr, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(term, base + o_t, b_node, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && bispec) e = cudaMemcpyAsync(bispec, base + o_b, b_node, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return tp_cuda(ctx, e, "bkappa nodes");
}

// ---------------------------------------------------------------------------
// <Map^3>
// ---------------------------------------------------------------------------
static const int MAP3_MAX_SWEEPS = 2000;
static const size_t MAP3_ESCALATE_BYTES = size_t(32) << 30;

extern "C" int tp_ctx_set_limits(tp_ctx* ctx, int region_cap, int max_ctas) {
  if (!ctx || region_cap < 64 || max_ctas < 0) return TP_ERR_ARG;
  ctx->region_cap = region_cap;
  ctx->max_ctas = max_ctas;
  return TP_OK;
}

extern "C" int tp_ctx_set_escalation(tp_ctx* ctx, int max_region_cap) {
  if (!ctx || max_region_cap < 0) return TP_ERR_ARG;
  ctx->escalate_cap = max_region_cap;
  return TP_OK;
}

extern "C" int tp_ctx_set_map3_cluster(tp_ctx* ctx, int on) {
  if (!ctx || on < 0 || on > 2) return TP_ERR_ARG;
  ctx->map3_cluster = on;
  return TP_OK;
}

extern "C" int tp_map3_jobs_device(tp_ctx* ctx, const int* job_cosmo, const double* job_theta, int n_jobs,
                                   double phi_min, double phi_max, double l_min, double l_max, double rel_tol,
                                   int precision, double* out, double* err, int64_t* neval, int64_t* nlive,
                                   int* status, const int* job_order) {
  TpRange nvtx_range("tp_map3_jobs_device: <Map^3> launch");
  if (!ctx || !job_cosmo || !job_theta || !out || n_jobs < 0) return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  if (!(rel_tol > 0) || !(phi_max > phi_min) || !(l_min >= 0)) return TP_ERR_ARG;
  if (ctx->n_cosmo == 0) return tp_fail(ctx, TP_ERR_STATE, "no cosmology set");
  if (n_jobs == 0) return TP_OK;
  cudaSetDevice(ctx->device);
  int grid = 0, cluster = 1;
  size_t smem = 0, scratch = 0;
  cudaError_t e = plan_map3(precision, n_jobs, ctx->region_cap, ctx->max_ctas, ctx->map3_cluster, &grid, &cluster,
                            &smem, &scratch);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "map3 plan");
  int st = ctx->ensure_scratch(scratch);
  if (st) return st;
  Map3Launch L;
  L.precision = precision;
  L.njobs = n_jobs;
  L.job_cosmo = job_cosmo;
  L.job_theta = job_theta;
  L.ncoef64 = ctx->d_ncoef64;
  L.ncoef32 = ctx->d_ncoef32;
  L.fcoef32 = ctx->d_fcoef32;
  L.wscale64 = ctx->d_wscale64;
  L.wscale32 = ctx->d_wscale32;
  L.ck64 = ctx->d_ck64;
  L.ck32 = ctx->d_ck32;
  L.lmin = l_min;
  L.lmax = l_max;
  L.phimin = phi_min;
  L.phimax = phi_max;
  L.rel_tol = rel_tol;
  L.cap = ctx->region_cap;
  L.max_sweeps = MAP3_MAX_SWEEPS;
  L.out = out;
  L.err = err;
  L.neval = neval;
  L.nlive = nlive;
  L.status = status;
  L.job_counter = ctx->d_counter;
  L.diag = ctx->d_diag;
  L.job_order = job_order;
  L.cluster = cluster;
  e = launch_map3(L, grid, smem, ctx->d_scratch, ctx->stream);
  return tp_cuda(ctx, e, "map3 launch");
}

extern "C" int tp_map3_batch(tp_ctx* ctx, const int* cosmo_index, int n_cosmo, const double* thetas, int n_trip,
                             double phi_min, double phi_max, double l_min, double l_max, double rel_tol,
                             int precision, double* out, double* err, int64_t* neval, int* status_out) {
  TpRange nvtx_range("tp_map3_batch: <Map^3>");
  if (!ctx || !thetas || !out || n_cosmo <= 0 || n_trip <= 0) return TP_ERR_ARG;
  if (ctx->n_cosmo == 0) return tp_fail(ctx, TP_ERR_STATE, "no cosmology set");
  for (int t = 0; t < 3 * n_trip; ++t)
    if (!(thetas[t] > 0)) return tp_fail(ctx, TP_ERR_ARG, "aperture radii must be > 0");
  std::vector<int> cidx(n_cosmo);
  for (int c = 0; c < n_cosmo; ++c) {
    cidx[c] = cosmo_index ? cosmo_index[c] : c;
    if (cidx[c] < 0 || cidx[c] >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_ARG, "bad cosmology index");
  }
  const int nj = n_cosmo * n_trip;
  std::vector<int> jc(nj);
  std::vector<double> jt(3 * (size_t)nj);
  for (int c = 0; c < n_cosmo; ++c)
    for (int t = 0; t < n_trip; ++t) {
      int j = c * n_trip + t;
      jc[j] = cidx[c];
      for (int q = 0; q < 3; ++q) jt[3 * (size_t)j + q] = thetas[3 * t + q];
    }
  // longest-first order from the costs seen for the same triplets before
  // (unseen triplets first); costs barely depend on the cosmology
  std::vector<std::string> keys(n_trip);
  std::vector<double> pred(n_trip);
  for (int t = 0; t < n_trip; ++t) {
    char buf[128];
    snprintf(buf, sizeof(buf), "%a,%a,%a,%a,%a,%a,%a,%a,%d", thetas[3 * t], thetas[3 * t + 1], thetas[3 * t + 2],
             phi_min, phi_max, l_min, l_max, rel_tol, precision);
    keys[t] = buf;
    auto it = ctx->map3_cost.find(keys[t]);
    pred[t] = it == ctx->map3_cost.end() ? 1e300 : it->second;
  }
  std::vector<int> order(nj);
  for (int j = 0; j < nj; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return pred[a % n_trip] > pred[b % n_trip]; });
  cudaSetDevice(ctx->device);
  size_t o_th = 0, o_c = (sizeof(double) * 3 * nj + 255) & ~size_t(255);
  size_t o_out = o_c + ((sizeof(int) * nj + 255) & ~size_t(255));
  size_t o_err = o_out + ((sizeof(double) * nj + 255) & ~size_t(255));
  size_t o_nev = o_err + ((sizeof(double) * nj + 255) & ~size_t(255));
  size_t o_st = o_nev + ((sizeof(int64_t) * nj + 255) & ~size_t(255));
  size_t o_ord = o_st + ((sizeof(int) * nj + 255) & ~size_t(255));
  size_t total = o_ord + sizeof(int) * nj + 256;
  int st = ctx->ensure_io(total);
  if (st) return st;
  char* b = ctx->d_io;
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(b + o_th, jt.data(), sizeof(double) * 3 * nj, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_c, jc.data(), sizeof(int) * nj, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_ord, order.data(), sizeof(int) * nj, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "map3 upload");
  st = tp_map3_jobs_device(ctx, (int*)(b + o_c), (double*)(b + o_th), nj, phi_min, phi_max, l_min, l_max, rel_tol,
                           precision, (double*)(b + o_out), (double*)(b + o_err), (int64_t*)(b + o_nev), nullptr,
                           (int*)(b + o_st), (int*)(b + o_ord));
  if (st) return st;
  std::vector<int> hst(nj);
  std::vector<int64_t> hnev(nj);
  e = cudaMemcpyAsync(out, b + o_out, sizeof(double) * nj, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && err) e = cudaMemcpyAsync(err, b + o_err, sizeof(double) * nj, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hnev.data(), b + o_nev, sizeof(int64_t) * nj, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hst.data(), b + o_st, sizeof(int) * nj, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "map3");
  // integrals that reached the region cap: integrated again, from the start,
  // with 16x the cap on as many CTAs as fit MAP3_ESCALATE_BYTES of region
  // stores, up to ctx->escalate_cap (the reference's hcubature_v has no cap;
  // the adaptive sequence is deterministic, so the larger cap continues where
  // the smaller one stopped)
  for (int cap = ctx->region_cap; cap < ctx->escalate_cap;) {
    std::vector<int> again;
    for (int j = 0; j < nj; ++j)
      if (hst[j] & 1) again.push_back(j);
    if (again.empty()) break;
    cap = (int)std::min<long>((long)cap * 16, ctx->escalate_cap);
    const int na = (int)again.size();
    std::vector<int> ac(na);
    std::vector<double> at(3 * (size_t)na);
    for (int k = 0; k < na; ++k) {
      ac[k] = jc[again[k]];
      for (int q = 0; q < 3; ++q) at[3 * (size_t)k + q] = jt[3 * (size_t)again[k] + q];
    }
    e = cudaMemcpyAsync(b + o_th, at.data(), sizeof(double) * 3 * na, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_c, ac.data(), sizeof(int) * na, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp_cuda(ctx, e, "map3 escalation upload");
    const int saved_cap = ctx->region_cap, saved_ctas = ctx->max_ctas;
    ctx->region_cap = cap;
    ctx->max_ctas = (int)std::max<size_t>(1, MAP3_ESCALATE_BYTES / Slot<3, 1>::bytes(cap));
    if (saved_ctas > 0) ctx->max_ctas = std::min(ctx->max_ctas, saved_ctas);
    st = tp_map3_jobs_device(ctx, (int*)(b + o_c), (double*)(b + o_th), na, phi_min, phi_max, l_min, l_max, rel_tol,
                             precision, (double*)(b + o_out), (double*)(b + o_err), (int64_t*)(b + o_nev), nullptr,
                             (int*)(b + o_st), nullptr);
    ctx->region_cap = saved_cap;
    ctx->max_ctas = saved_ctas;
    if (st) return st;
    std::vector<double> ao(na), ae(na);
    std::vector<int64_t> an(na);
    std::vector<int> as(na);
    e = cudaMemcpyAsync(ao.data(), b + o_out, sizeof(double) * na, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ae.data(), b + o_err, sizeof(double) * na, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(an.data(), b + o_nev, sizeof(int64_t) * na, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(as.data(), b + o_st, sizeof(int) * na, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return tp_cuda(ctx, e, "map3 escalation");
    for (int k = 0; k < na; ++k) {
      const int j = again[k];
      out[j] = ao[k];
      if (err) err[j] = ae[k];
      hnev[j] = an[k];
      hst[j] = as[k];
    }
  }
  if (ctx->scratch_bytes > (size_t(4) << 30)) {  // region stores grown by the escalation are released
    cudaFree(ctx->d_scratch);
    ctx->d_scratch = nullptr;
    ctx->scratch_bytes = 0;
  }
  if (neval) memcpy(neval, hnev.data(), sizeof(int64_t) * nj);
  for (int t = 0; t < n_trip; ++t) {
    double m = 0;
    for (int c = 0; c < n_cosmo; ++c) m += (double)hnev[c * n_trip + t];
    ctx->map3_cost[keys[t]] = m / n_cosmo;
  }
  int bad = 0;
  for (int j = 0; j < nj; ++j) {
    if (status_out) status_out[j] = hst[j];
    if (hst[j]) ++bad;
  }
  if (bad) return tp_fail(ctx, TP_ERR_CAPACITY, std::to_string(bad) + " integrals hit a region or sweep cap");
  return TP_OK;
}
