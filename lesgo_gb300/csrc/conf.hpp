// lesgo.conf reader (input_util.f90:54-1023) and turbine placement
// (turbines.f90:740-866), host side.
//
// Grammar as the reference reads it: every line loses all blanks and tabs
// (string_util.f90:125-154); blank lines and lines starting with '!' are
// skipped; a line holding '{' opens the block named before it; '}' closes
// it; inside a block every line is KEY=value (no '=' or nothing after it is
// an error).  Keys and block names are case-insensitive.  Values are read
// list-directed: the text up to the first ',' or '/' is the value; logicals
// take T/F after an optional '.'; reals accept a D exponent.  Unknown keys
// are reported and ignored; blocks of features this library leaves out
// (LEVEL_SET, SCALARS, and TURBINES when turbines are not used) are skipped
// to their closing brace like the reference does for blocks it was built
// without.  Settings that would change the time step in ways this library
// does not implement are rejected with LESGO_ERR_UNSUPPORTED.
#pragma once

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "lesgo_gpu.h"

namespace lesgo {
namespace conf {

struct ConfError {
  int code;
  std::string msg;
};

struct Turbines {
  int num_x = 0, num_y = 0, orientation = 1;
  double dia_all = 0, height_all = 0, thk_all = 0, stag_perc = 0, theta1_all = 0, theta2_all = 0;
  double Ct_prime = 1.33;
  bool read_param = false, dyn_theta1 = false, dyn_theta2 = false, dyn_Ct_prime = false, use_rotation = false;
};

static std::string upper(std::string s) {
  for (char& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

struct Reader {
  std::string file;
  int line = 0;
  std::string log;

  [[noreturn]] void fail(int code, const std::string& m) const {
    throw ConfError{code, file + ":" + std::to_string(line) + ": " + m};
  }
  static std::string token(const std::string& v) {
    const size_t e = v.find_first_of(",/");
    return e == std::string::npos ? v : v.substr(0, e);
  }
  int as_int(const std::string& v) const {
    const std::string t = token(v);
    char* end;
    const long x = std::strtol(t.c_str(), &end, 10);
    if (t.empty() || *end != '\0') fail(LESGO_ERR_ARG, "not an integer: " + v);
    return (int)x;
  }
  double as_real(const std::string& v) const {
    std::string t = token(v);
    for (char& c : t)
      if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
    char* end;
    const double x = std::strtod(t.c_str(), &end);
    if (t.empty() || *end != '\0') fail(LESGO_ERR_ARG, "not a real: " + v);
    return x;
  }
  bool as_bool(const std::string& v) const {
    std::string t = token(v);
    size_t i = (!t.empty() && t[0] == '.') ? 1 : 0;
    if (i < t.size()) {
      const char c = (char)std::toupper((unsigned char)t[i]);
      if (c == 'T') return true;
      if (c == 'F') return false;
    }
    fail(LESGO_ERR_ARG, "not a logical: " + v);
  }
};

// Reference defaults of the parameters read (param.f90:100-240,
// sgs_param.f90) in lesgo_params_t / lesgo_run_t.
static void defaults(lesgo_params_t* p, lesgo_run_t* r) {
  lesgo_gpu_params_default(p);
  const double pi = 3.1415926535897932384626433;
  p->nx = 64; p->ny = 64; p->nz_tot = 64;
  p->z_i = 1000.0;
  p->L_x = 2.0 * pi; p->L_y = 2.0 * pi; p->L_z = 1.0;
  p->sgs_model = 5; p->cs_count = 5; p->dyn_init = 100; p->ifilter = 1;
  p->u_star = 0.45; p->vonk = 0.4; p->nu_molec = 1.14e-5; p->molec = 0;
  p->dt = 2.0e-4;
  p->initu = 0; p->lbc_mom = 1; p->ubc_mom = 0; p->ubot = 0.0; p->utop = 0.0; p->zo = 0.0001;
  p->use_mean_p_force = 1; p->eval_mean_p_force = 0; p->mean_p_force_x = 1.0; p->mean_p_force_y = 0.0;
  p->n_turbines = 0; p->turbines = nullptr;
  r->nproc = 1; r->uniform_spacing = 0; r->wall_damp_exp = 2; r->Co = 0.16; r->sgs = 1;
  r->nsteps = 50000; r->runtime = -1; r->use_cfl_dt = 0;
  r->cfl = p->cfl = (double)0.05f;   // param.f90: a default-real literal
  p->use_cfl_dt = 0;
  r->cumulative_time = 1; r->inilag = 1;
  r->wbase = 100; r->nenergy = 100; r->lag_cfl_count = 1000;
  r->checkpoint_data = 0; r->checkpoint_nskip = 10000;
  r->tavg_calc = 0; r->tavg_nstart = 1; r->tavg_nend = 50000; r->tavg_nskip = 100;
}

// turbines.f90:740-866: positions, sizes and yaw of num_x * num_y disks, in
// units of z_i.  `param_dat` is read when read_param is set.
static std::vector<lesgo_turbine_t> place(const Turbines& t, const lesgo_params_t& p, const std::string& param_dat) {
  const int nloc = t.num_x * t.num_y;
  std::vector<lesgo_turbine_t> w(nloc);
  if (nloc <= 0) return w;
  const double z_i = p.z_i;
  if (t.read_param) {
    FILE* f = std::fopen(param_dat.c_str(), "r");
    if (!f) throw ConfError{LESGO_ERR_ARG, "file " + param_dat + " does not exist"};
    std::vector<std::vector<double>> rows;
    char buf[4096];
    while (std::fgets(buf, sizeof buf, f)) {
      std::string s(buf);
      for (char& c : s)
        if (c == ',' || c == '\t' || c == '\r' || c == '\n') c = ' ';
      for (char& c : s)
        if (c == 'd' || c == 'D') c = 'e';
      std::vector<double> v;
      const char* q = s.c_str();
      char* end;
      for (;;) {
        const double x = std::strtod(q, &end);
        if (end == q) break;
        v.push_back(x);
        q = end;
      }
      if (!v.empty()) rows.push_back(v);
    }
    std::fclose(f);
    if ((int)rows.size() < nloc) throw ConfError{LESGO_ERR_ARG, param_dat + " must have num_x*num_y lines"};
    for (int k = 0; k < nloc; ++k) {
      if (rows[k].size() < 8) throw ConfError{LESGO_ERR_ARG, param_dat + ": 8 values per line expected"};
      const std::vector<double>& r = rows[k];
      w[k].xloc = r[0] / z_i; w[k].yloc = r[1] / z_i; w[k].height = r[2] / z_i;
      w[k].dia = r[3] / z_i; w[k].thk = r[4] / z_i;
      w[k].theta1 = r[5]; w[k].theta2 = r[6]; w[k].Ct_prime = r[7];
    }
    return w;
  }
  const double height_all = t.height_all / z_i, dia_all = t.dia_all / z_i, thk_all = t.thk_all / z_i;
  const double sx = p.L_x / (t.num_x * dia_all), sy = p.L_y / (t.num_y * dia_all);
  const double sxx = sx * dia_all, syy = sy * dia_all;
  for (auto& x : w) {
    x.height = height_all; x.dia = dia_all; x.thk = thk_all;
    x.theta1 = t.theta1_all; x.theta2 = t.theta2_all; x.Ct_prime = t.Ct_prime;
  }
  int k = 0;
  for (int i = 1; i <= t.num_x; ++i)
    for (int j = 1; j <= t.num_y; ++j, ++k) {
      w[k].xloc = sxx * (double)((float)(2 * i - 1) / 2.0f);
      w[k].yloc = syy * (double)((float)(2 * j - 1) / 2.0f);
    }
  const double pct = t.stag_perc / 100.0;
  switch (t.orientation) {
    case 1: break;
    case 2:
      for (int i = 2; i <= t.num_x; ++i)
        for (int q = 1 + t.num_y * (i - 1); q <= t.num_y * i; ++q) {
          const double shift_base = syy * pct;
          w[q - 1].yloc = std::fmod(w[q - 1].yloc + (i - 1) * shift_base, p.L_y);
        }
      break;
    case 3:
      for (int i = 2; i <= t.num_x; i += 2)
        for (int q = 1 + t.num_y * (i - 1); q <= t.num_y * i; ++q) w[q - 1].height = height_all * (1. + pct);
      for (int i = 1; i <= t.num_x; i += 2)
        for (int q = 1 + t.num_y * (i - 1); q <= t.num_y * i; ++q) w[q - 1].height = height_all * (1. - pct);
      break;
    case 4: {
      int q = 0;
      for (int i = 1; i <= t.num_x; ++i)
        for (int j = 1; j <= t.num_y; ++j, ++q) {
          const double c = 2. * std::fmod((double)(i + j), 2.) - 1.;
          w[q].height = height_all * (1. + c * pct);
        }
      break;
    }
    case 5: {
      if (nloc < 2) throw ConfError{LESGO_ERR_ARG, "orientation 5 needs at least two turbines"};
      const double dummy = t.stag_perc * (w[1].yloc - w[0].yloc);
      int q = 0;
      for (int i = 1; i <= t.num_x; ++i)
        for (int j = 1; j <= t.num_y; ++j, ++q) w[q].yloc = std::fmod(w[q].yloc + dummy * (i - 1), p.L_y);
      break;
    }
    default: throw ConfError{LESGO_ERR_ARG, "invalid orientation"};
  }
  return w;
}

// Read <path>lesgo.conf.  Turbines go to `tbuf` (capacity `tmax`); with
// `with_turbines` zero the TURBINES block is skipped.
static void read(const std::string& path, int with_turbines, lesgo_params_t* p, lesgo_run_t* r,
                 lesgo_turbine_t* tbuf, int tmax, std::string* log) {
  defaults(p, r);
  Reader rd;
  rd.file = path + "lesgo.conf";
  FILE* f = std::fopen(rd.file.c_str(), "r");
  if (!f) throw ConfError{LESGO_ERR_ARG, "file " + rd.file + " does not exist"};
  std::vector<std::string> lines;
  {
    std::string cur;
    int c;
    while ((c = std::fgetc(f)) != EOF) {
      if (c == '\n') { lines.push_back(cur); cur.clear(); }
      else cur.push_back((char)c);
    }
    if (!cur.empty()) lines.push_back(cur);
    std::fclose(f);
  }
  size_t li = 0;
  // readline (input_util.f90:900-935): next line with content, blanks removed
  auto next = [&](std::string& buf) -> bool {
    while (li < lines.size()) {
      std::string s;
      for (char c : lines[li])
        if (c != ' ' && c != '\t' && c != '\r') s.push_back(c);
      ++li;
      rd.line = (int)li;
      if (s.empty() || s[0] == '!') continue;
      buf = s;
      return true;
    }
    return false;
  };
  Turbines tb;
  bool seen_turbines = false;
  std::string buf;
  auto note = [&](const std::string& m) { rd.log += m + "\n"; };
  while (next(buf)) {
    const size_t be = buf.find('{');
    if (be == std::string::npos) rd.fail(LESGO_ERR_ARG, "block entry not found");
    const std::string block = upper(buf.substr(0, be));
    const bool known = block == "DOMAIN" || block == "MODEL" || block == "CORIOLIS" || block == "TIME" ||
                       block == "FLOW_COND" || block == "OUTPUT" || (block == "TURBINES" && with_turbines);
    if (!known) {
      note("Found unused input block: " + block);
      bool closed = buf.find('}') != std::string::npos;
      while (!closed && next(buf)) closed = buf.find('}') != std::string::npos;
      continue;
    }
    if (block == "TURBINES") seen_turbines = true;
    for (;;) {
      if (!next(buf)) rd.fail(LESGO_ERR_ARG, "Bad read in block " + block);
      const size_t bx = buf.find('}'), eq = buf.find('=');
      if (bx == 0) break;
      if (bx != std::string::npos) rd.fail(LESGO_ERR_ARG, block + " data block not formatted correctly: " + buf);
      if (eq == std::string::npos) rd.fail(LESGO_ERR_ARG, "Bad read in block at line: " + buf);
      if (eq + 1 == buf.size()) rd.fail(LESGO_ERR_ARG, "nothing after equals sign");
      const std::string key = upper(buf.substr(0, eq)), v = buf.substr(eq + 1);
      bool used = true;
      if (block == "DOMAIN") {
        if (key == "NPROC") r->nproc = rd.as_int(v);
        else if (key == "NX") p->nx = rd.as_int(v);
        else if (key == "NY") p->ny = rd.as_int(v);
        else if (key == "NZ") p->nz_tot = rd.as_int(v);
        else if (key == "Z_I") p->z_i = rd.as_real(v);
        else if (key == "LX") p->L_x = rd.as_real(v);
        else if (key == "LY") p->L_y = rd.as_real(v);
        else if (key == "LZ") p->L_z = rd.as_real(v);
        else if (key == "UNIFORM_SPACING") r->uniform_spacing = rd.as_bool(v);
        else used = false;
      } else if (block == "MODEL") {
        if (key == "SGS_MODEL") p->sgs_model = rd.as_int(v);
        else if (key == "WALL_DAMP_EXP") r->wall_damp_exp = rd.as_int(v);
        else if (key == "CS_COUNT") p->cs_count = rd.as_int(v);
        else if (key == "DYN_INIT") p->dyn_init = rd.as_int(v);
        else if (key == "CO") r->Co = rd.as_real(v);
        else if (key == "IFILTER") p->ifilter = rd.as_int(v);
        else if (key == "U_STAR") p->u_star = rd.as_real(v);
        else if (key == "VONK") p->vonk = rd.as_real(v);
        else if (key == "NU_MOLEC") p->nu_molec = rd.as_real(v);
        else if (key == "MOLEC") p->molec = rd.as_bool(v);
        else if (key == "SGS") r->sgs = rd.as_bool(v);
        else used = false;
      } else if (block == "CORIOLIS") {
        if (key == "CORIOLIS_FORCING") {
          if (rd.as_int(v) != 0) rd.fail(LESGO_ERR_UNSUPPORTED, "coriolis_forcing other than 0");
        } else if (key == "FC" || key == "G" || key == "ALPHA" || key == "PID_TIME" || key == "PHI_SET" ||
                   key == "HEIGHT_SET" || key == "KP" || key == "KI" || key == "KD" || key == "REPEAT_INTERVAL") {
        } else used = false;
      } else if (block == "TIME") {
        if (key == "NSTEPS") r->nsteps = rd.as_int(v);
        else if (key == "RUNTIME") r->runtime = rd.as_int(v);
        else if (key == "USE_CFL_DT") r->use_cfl_dt = p->use_cfl_dt = rd.as_bool(v);
        else if (key == "CFL") r->cfl = p->cfl = rd.as_real(v);
        else if (key == "DT") p->dt = rd.as_real(v);
        else if (key == "CUMULATIVE_TIME") r->cumulative_time = rd.as_bool(v);
        else used = false;
      } else if (block == "FLOW_COND") {
        if (key == "INITU") p->initu = rd.as_bool(v);
        else if (key == "INILAG") r->inilag = rd.as_bool(v);
        else if (key == "LBC_MOM") p->lbc_mom = rd.as_int(v);
        else if (key == "UBC_MOM") p->ubc_mom = rd.as_int(v);
        else if (key == "UBOT") p->ubot = rd.as_real(v);
        else if (key == "UTOP") p->utop = rd.as_real(v);
        else if (key == "USE_SPONGE") {
          if (rd.as_bool(v)) rd.fail(LESGO_ERR_UNSUPPORTED, "use_sponge");
        } else if (key == "ZO") p->zo = rd.as_real(v);
        else if (key == "INFLOW_TYPE") {
          if (rd.as_int(v) != 0) rd.fail(LESGO_ERR_UNSUPPORTED, "inflow_type other than 0");
        } else if (key == "USE_MEAN_P_FORCE") p->use_mean_p_force = rd.as_bool(v);
        else if (key == "EVAL_MEAN_P_FORCE") p->eval_mean_p_force = rd.as_bool(v);
        else if (key == "MEAN_P_FORCE_X") p->mean_p_force_x = rd.as_real(v);
        else if (key == "MEAN_P_FORCE_Y") p->mean_p_force_y = rd.as_real(v);
        else if (key == "USE_RANDOM_FORCE") {
          if (rd.as_bool(v)) rd.fail(LESGO_ERR_UNSUPPORTED, "use_random_force");
        } else if (key == "SPONGE_FREQUENCY" || key == "SPONGE_HEIGHT" || key == "FRINGE_REGION_END" ||
                   key == "FRINGE_REGION_LEN" || key == "INFLOW_VELOCITY" || key == "SAMPLING_REGION_END" ||
                   key == "SHIFT_N" || key == "STOP_RANDOM_FORCE" || key == "RMS_RANDOM_FORCE" || key == "UP_IN" ||
                   key == "TI_OUT" || key == "LX_HIT" || key == "LY_HIT" || key == "LZ_HIT" || key == "NX_HIT" ||
                   key == "NY_HIT" || key == "NZ_HIT" || key == "U_FILE" || key == "V_FILE" || key == "W_FILE") {
        } else used = false;
      } else if (block == "OUTPUT") {
        if (key == "WBASE") r->wbase = rd.as_int(v);
        else if (key == "NENERGY") r->nenergy = rd.as_int(v);
        else if (key == "LAG_CFL_COUNT") r->lag_cfl_count = rd.as_int(v);
        else if (key == "CHECKPOINT_DATA") r->checkpoint_data = rd.as_bool(v);
        else if (key == "CHECKPOINT_NSKIP") r->checkpoint_nskip = rd.as_int(v);
        else if (key == "TAVG_CALC") r->tavg_calc = rd.as_bool(v);
        else if (key == "TAVG_NSTART") r->tavg_nstart = rd.as_int(v);
        else if (key == "TAVG_NEND") r->tavg_nend = rd.as_int(v);
        else if (key == "TAVG_NSKIP") r->tavg_nskip = rd.as_int(v);
        else {
          static const char* io[] = {"POINT", "DOMAIN", "XPLANE", "YPLANE", "ZPLANE"};
          used = false;
          for (const char* pre : io) {
            const std::string ps(pre);
            if (key.compare(0, ps.size() + 1, ps + "_") == 0) used = true;
          }
        }
      } else if (block == "TURBINES") {
        if (key == "NUM_X") tb.num_x = rd.as_int(v);
        else if (key == "NUM_Y") tb.num_y = rd.as_int(v);
        else if (key == "DIA_ALL") tb.dia_all = rd.as_real(v);
        else if (key == "HEIGHT_ALL") tb.height_all = rd.as_real(v);
        else if (key == "THK_ALL") tb.thk_all = rd.as_real(v);
        else if (key == "ORIENTATION") tb.orientation = rd.as_int(v);
        else if (key == "STAG_PERC") tb.stag_perc = rd.as_real(v);
        else if (key == "THETA1_ALL") tb.theta1_all = rd.as_real(v);
        else if (key == "THETA2_ALL") tb.theta2_all = rd.as_real(v);
        else if (key == "CT_PRIME") tb.Ct_prime = rd.as_real(v);
        else if (key == "READ_PARAM") tb.read_param = rd.as_bool(v);
        else if (key == "DYN_THETA1") tb.dyn_theta1 = rd.as_bool(v);
        else if (key == "DYN_THETA2") tb.dyn_theta2 = rd.as_bool(v);
        else if (key == "DYN_CT_PRIME") tb.dyn_Ct_prime = rd.as_bool(v);
        else if (key == "USE_ROTATION") tb.use_rotation = rd.as_bool(v);
        else if (key == "T_AVG_DIM") p->T_avg_dim = rd.as_real(v);
        else if (key == "ALPHA1") p->alpha1 = rd.as_real(v);
        else if (key == "ALPHA2") p->alpha2 = rd.as_real(v);
        else if (key == "FILTER_CUTOFF") p->filter_cutoff = rd.as_real(v);
        else if (key == "ADM_CORRECTION") p->adm_correction = rd.as_bool(v);
        else if (key == "TIP_SPEED_RATIO" || key == "TBASE") {
        } else used = false;
      }
      if (!used) note("Found unused data value in " + block + " block: " + key);
    }
  }
  // domain_block's derived values (input_util.f90:196-235)
  if (p->nx < 1 || p->ny < 1 || p->nz_tot < 1) throw ConfError{LESGO_ERR_ARG, "Nx, Ny, Nz must be positive"};
  if (r->uniform_spacing) {
    const int nz = p->nz_tot + 1;   // one process
    const double dx = p->L_x / p->nx;
    p->L_y = p->ny * dx;
    p->L_z = (nz - 1) * dx;
  }
  if (!r->sgs) throw ConfError{LESGO_ERR_UNSUPPORTED, "sgs = .false. (no SGS model)"};
  if (seen_turbines) {
    r->dyn_theta1 = tb.dyn_theta1; r->dyn_theta2 = tb.dyn_theta2; r->dyn_ct_prime = tb.dyn_Ct_prime;
    if (tb.use_rotation) throw ConfError{LESGO_ERR_UNSUPPORTED, "use_rotation"};
    const std::vector<lesgo_turbine_t> w = place(tb, *p, path + "input_turbines/param.dat");
    if ((int)w.size() > tmax) throw ConfError{LESGO_ERR_ARG, "turbine buffer holds fewer than num_x*num_y disks"};
    for (size_t k = 0; k < w.size(); ++k) tbuf[k] = w[k];
    p->n_turbines = (int)w.size();
    p->turbines = w.empty() ? nullptr : tbuf;
  }
  if (log) *log = rd.log;
}

// read_control_files (turbines.f90:872-931): every non-blank line of the
// file is one row, the dimensional time then one value per turbine
// (list-directed: blanks or commas between values, D exponents).
static std::vector<double> read_schedule(const std::string& path, int which, int nturb) {
  static const char* names[] = {"theta1.dat", "theta2.dat", "Ct_prime.dat"};
  if (which < 0 || which > 2 || nturb < 1) throw ConfError{LESGO_ERR_ARG, "bad schedule request"};
  const std::string file = path + "input_turbines/" + names[which];
  FILE* f = std::fopen(file.c_str(), "r");
  if (!f) throw ConfError{LESGO_ERR_ARG, "file " + file + " does not exist"};
  std::vector<double> rows;
  std::string s;
  int line = 0;
  for (int c = 0; c != EOF;) {
    s.clear();
    while ((c = std::fgetc(f)) != EOF && c != '\n') s.push_back((char)c);
    ++line;
    for (char& ch : s)
      if (ch == ',' || ch == '\t' || ch == '\r') ch = ' ';
      else if (ch == 'd' || ch == 'D') ch = 'e';
    std::vector<double> v;
    const char* q = s.c_str();
    char* end;
    for (;;) {
      const double x = std::strtod(q, &end);
      if (end == q) break;
      v.push_back(x);
      q = end;
    }
    while (*q == ' ') ++q;
    if (v.empty() && *q == '\0') continue;
    if ((int)v.size() < 1 + nturb || *q != '\0') {
      std::fclose(f);
      throw ConfError{LESGO_ERR_ARG, file + ":" + std::to_string(line) + ": expected the time and " +
                                         std::to_string(nturb) + " values"};
    }
    rows.insert(rows.end(), v.begin(), v.begin() + 1 + nturb);
  }
  std::fclose(f);
  if (rows.empty()) throw ConfError{LESGO_ERR_ARG, file + " holds no rows"};
  return rows;
}

}  // namespace conf
}  // namespace lesgo
