// The cosmosis module entry of the reference (cuda_version/interface.cu:16-257)
// on top of the C ABI: setup / execute / cleanup with the same section, keys,
// triplet enumeration, P(k) conversion and outputs. The data block is reached
// through the tp_datablock callback table (include/threepoint_gb300_module.h),
// so cosmosis is not a build dependency.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <map>
#include <string>
#include <vector>

#include "threepoint_gb300.h"
#include "threepoint_gb300_module.h"

struct tp_module {
  int device = 0;
  double zmax = 0;
  std::vector<double> nz;  // 256 bins
  std::vector<double> th;  // [n][3] rad
  bool output = false;
  std::string output_dir;
  tp_ctx* ctx = nullptr;
  int precision = TP_FP64;
  std::string err;
};

static int fail(tp_module* m, int st, const std::string& msg) {
  m->err = msg;
  return st;
}

extern "C" const char* tp_module_last_error(const tp_module* m) { return m ? m->err.c_str() : "null module"; }

// theta triplets of setup (interface.cu:103-133): theta_bins log-spaced radii
// between theta_min and theta_max; all theta1 <= theta2 <= theta3, or only the
// equal ones
static void build_triplets(double tmin, double tmax, int nbins, bool diag, std::vector<double>& th) {
  const double dl = (log(tmax) - log(tmin)) / (nbins - 1);
  for (int i = 0; i < nbins; i++) {
    const double t1 = tmin * exp(i * dl);
    if (diag) {
      th.insert(th.end(), {t1, t1, t1});
      continue;
    }
    for (int j = i; j < nbins; j++) {
      const double t2 = tmin * exp(j * dl);
      for (int k = j; k < nbins; k++) th.insert(th.end(), {t1, t2, tmin * exp(k * dl)});
    }
  }
}

static int read_setup(tp_module* m, const tp_datablock* o) {
  const char* sec = "threepoint";
  char buf[4096];
  if (o->get_string(o->handle, sec, "nz_file", buf, sizeof(buf)))
    return fail(m, TP_ERR_FORMAT, "threepoint/nz_file missing");
  const std::string fn_nz = buf;
  if (o->get_double(o->handle, sec, "zMax", &m->zmax)) return fail(m, TP_ERR_FORMAT, "threepoint/zMax missing");
  m->nz.assign(256, 0.0);
  int st = tp_read_n_of_z(fn_nz.c_str(), 256, m->zmax, m->nz.data());
  if (st) return fail(m, st, "could not read n(z) from " + fn_nz);
  if (o->get_string(o->handle, sec, "theta_unit", buf, sizeof(buf)))
    return fail(m, TP_ERR_FORMAT, "threepoint/theta_unit missing");
  const std::string unit = buf;
  double tmin, tmax;
  int nbins, diag, outp;
  if (o->get_double(o->handle, sec, "theta_min", &tmin) || o->get_double(o->handle, sec, "theta_max", &tmax) ||
      o->get_int(o->handle, sec, "theta_bins", &nbins) || o->get_int(o->handle, sec, "diag_only", &diag))
    return fail(m, TP_ERR_FORMAT, "threepoint/theta_min, theta_max, theta_bins or diag_only missing");
  if (tp_convert_angle_to_rad(tmin, unit.c_str(), &tmin) || tp_convert_angle_to_rad(tmax, unit.c_str(), &tmax))
    return fail(m, TP_ERR_ARG, "theta_unit must be arcmin, deg or rad");
  // the reference divides by theta_bins - 1; one bin would give NaN radii
  if (nbins < 2 || !(tmin > 0) || !(tmax >= tmin)) return fail(m, TP_ERR_ARG, "need theta_bins >= 2, 0 < theta_min <= theta_max");
  build_triplets(tmin, tmax, nbins, diag != 0, m->th);
  if (o->get_int(o->handle, sec, "output_Map3", &outp) ||
      o->get_string(o->handle, sec, "output_dir", buf, sizeof(buf)))
    return fail(m, TP_ERR_FORMAT, "threepoint/output_Map3 or output_dir missing");
  m->output = outp != 0;
  m->output_dir = buf;
  return TP_OK;
}

extern "C" int tp_module_setup(const tp_datablock* options, int device, tp_module** out) {
  if (!options || !out || device < 0) return TP_ERR_ARG;
  *out = nullptr;
  tp_module* m = new tp_module();
  m->device = device;
  int st = read_setup(m, options);
  if (st) {
    fprintf(stderr, "threepoint_gb300 setup: %s\n", m->err.c_str());
    delete m;
    return st;
  }
  *out = m;
  return TP_OK;
}

// convert_Pk (helpers.cu:202-235): n log-spaced samples between the first and
// last k of the table, linear interpolation in k (valueMap, helpers.cu:217-235)
static void convert_pk(const std::map<double, double>& pk, int n, double& kmin, double& kmax, double& dk,
                       std::vector<double>& out) {
  kmin = pk.begin()->first;
  kmax = pk.rbegin()->first;
  dk = log(kmax / kmin) / n;
  out.clear();
  for (int i = 0; i < n; i++) {
    const double k = exp(log(kmin) + dk * i);
    auto hi = pk.upper_bound(k);
    double v;
    if (hi == pk.end()) {
      v = std::prev(hi)->second;
    } else if (hi == pk.begin()) {
      v = hi->second;
    } else {
      auto lo = std::prev(hi);
      const double d = (k - lo->first) / (hi->first - lo->first);
      v = d * hi->second + (1 - d) * lo->second;
    }
    out.push_back(v);
  }
}

extern "C" int tp_module_execute(tp_module* m, const tp_datablock* b) {
  if (!m || !b) return TP_ERR_ARG;
  const char* cs = "cosmological_parameters";
  tp_cosmology c;
  if (b->get_double(b->handle, cs, "omega_m", &c.om) || b->get_double(b->handle, cs, "sigma_8", &c.sigma8) ||
      b->get_double(b->handle, cs, "h0", &c.h) || b->get_double(b->handle, cs, "omega_b", &c.omb) ||
      b->get_double(b->handle, cs, "n_s", &c.ns) || b->get_double(b->handle, cs, "w", &c.w))
    return fail(m, TP_ERR_FORMAT, "cosmological_parameters incomplete");
  c.omc = c.om - c.omb;
  c.ow = 1 - c.om;
  c.zmax = m->zmax;

  int nk = 0, npk = 0, got = 0;
  if (b->get_double_array(b->handle, "matter_power_lin", "k_h", nullptr, 0, &nk) || nk < 2)
    return fail(m, TP_ERR_FORMAT, "matter_power_lin/k_h missing");
  if (b->get_double_array(b->handle, "matter_power_lin", "p_k", nullptr, 0, &npk) || npk < nk)
    return fail(m, TP_ERR_FORMAT, "matter_power_lin/p_k missing or shorter than k_h");
  std::vector<double> k(nk), pk(npk);
  if (b->get_double_array(b->handle, "matter_power_lin", "k_h", k.data(), nk, &got) ||
      b->get_double_array(b->handle, "matter_power_lin", "p_k", pk.data(), npk, &got))
    return fail(m, TP_ERR_FORMAT, "matter_power_lin unreadable");
  std::map<double, double> lin;
  for (int i = 0; i < nk; i++) lin[k[i]] = pk[i];  // P_k(0, i): first row (interface.cu:185-188)
  std::vector<double> pk256;
  double kmin, kmax, dk;
  convert_pk(lin, 256, kmin, kmax, dk, pk256);

  int st;
  if (!m->ctx && (st = tp_ctx_create(m->device, &m->ctx)) != TP_OK)
    return fail(m, st, std::string("CUDA context: ") + tp_status_string(st));
  st = tp_set_cosmologies(m->ctx, &c, 1, m->nz.data(), 0, pk256.data(), dk, kmin, kmax);
  if (st) return fail(m, st, tp_last_error(m->ctx));
  const int n = (int)(m->th.size() / 3);
  std::vector<double> map3(n);
  st = tp_map3_batch(m->ctx, nullptr, 1, m->th.data(), n, 0.0, 2 * M_PI, 1.0, 0.0, 1e-4, m->precision, map3.data(),
                     nullptr, nullptr, nullptr);
  if (st) return fail(m, st, tp_last_error(m->ctx));

  if (m->output) {  // interface.cu:199-212,227-233
    char name[128];
    snprintf(name, sizeof(name), "/om_%f_sig8_%f_h_%f_w_%f.dat", c.om, c.sigma8, c.h, c.w);
    const std::string fn = m->output_dir + name;
    std::ofstream o(fn);
    if (!o) return fail(m, TP_ERR_IO, "could not open " + fn);
    o << "#theta1[rad] theta2[rad] theta3[rad] Map^3" << std::endl;
    for (int i = 0; i < n; ++i)
      o << m->th[3 * i] << " " << m->th[3 * i + 1] << " " << m->th[3 * i + 2] << " " << map3[i] << std::endl;
  }
  if (b->put_double_array(b->handle, "threepoint", "Map3s", map3.data(), n))
    return fail(m, TP_ERR_IO, "could not write threepoint/Map3s");
  return TP_OK;
}

extern "C" int tp_module_cleanup(tp_module* m) {
  if (!m) return TP_ERR_ARG;
  if (m->ctx) tp_ctx_destroy(m->ctx);
  delete m;
  return TP_OK;
}

extern "C" int tp_module_set_precision(tp_module* m, int precision) {
  if (!m || (precision != TP_FP64 && precision != TP_FP32)) return TP_ERR_ARG;
  m->precision = precision;
  return TP_OK;
}

extern "C" int tp_module_n_triplets(const tp_module* m) { return m ? (int)(m->th.size() / 3) : 0; }

extern "C" int tp_module_triplets(const tp_module* m, double* out) {
  if (!m || !out) return TP_ERR_ARG;
  for (size_t i = 0; i < m->th.size(); ++i) out[i] = m->th[i];
  return TP_OK;
}
