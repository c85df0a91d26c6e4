// .ini front end of the library: the reference's ConfigMap semantics and
// HydroParams derivation, restated.
//   * inih line parsing: sections, name=value, ';' comments after whitespace,
//     '#'/';' comment lines, continuation lines replacing the value
//     (utils/config/inih/ini.cpp:80-160);
//   * keys are "section.name" lower-cased (INIReader.cpp:105-111);
//   * getFloat parses with strtof, so every real is rounded to float before it
//     becomes a double (ConfigMap.cpp:37-46); getInteger uses strtol base 0;
//   * HydroParams::HydroParams + init (HydroParams.cpp:37-180, 327-359).
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

#include "../../include/ek_gb300.h"
#include "ek_internal.h"

namespace
{

struct Ini
{
  std::map<std::string, std::string> values;
  int                                error_line = 0;
};

std::string
lower(std::string s)
{
  for (auto & c : s)
    c = (char)std::tolower((unsigned char)c);
  return s;
}

size_t
find_char_or_comment(const std::string & s, size_t from, char c)
{
  bool was_ws = false;
  size_t i = from;
  while (i < s.size() && s[i] != c && !(was_ws && s[i] == ';'))
  {
    was_ws = std::isspace((unsigned char)s[i]) != 0;
    ++i;
  }
  return i;
}

std::string
rstrip(const std::string & s)
{
  size_t e = s.size();
  while (e > 0 && std::isspace((unsigned char)s[e - 1]))
    --e;
  return s.substr(0, e);
}

Ini
parse(const char * text, size_t len)
{
  Ini         ini;
  std::string section, prev_name;
  size_t      pos = 0;
  int         lineno = 0;
  while (pos < len)
  {
    size_t eol = pos;
    while (eol < len && text[eol] != '\n')
      ++eol;
    // fgets with a 200-byte buffer keeps at most 199 characters per read
    std::string line(text + pos, std::min<size_t>(eol - pos, 199));
    pos = eol + 1;
    ++lineno;
    line = rstrip(line);
    size_t start = 0;
    while (start < line.size() && std::isspace((unsigned char)line[start]))
      ++start;
    if (!prev_name.empty() && start < line.size() && start > 0)
    {
      ini.values[lower(section + "." + prev_name)] = line.substr(start);
      continue;
    }
    if (start >= line.size() || line[start] == ';' || line[start] == '#')
      continue;
    if (line[start] == '[')
    {
      size_t end = find_char_or_comment(line, start + 1, ']');
      if (end < line.size() && line[end] == ']')
      {
        section = line.substr(start + 1, end - start - 1).substr(0, 49);
        prev_name.clear();
      }
      else if (!ini.error_line)
        ini.error_line = lineno;
      continue;
    }
    size_t end = find_char_or_comment(line, start, '=');
    if (end < line.size() && line[end] == '=')
    {
      std::string name = rstrip(line.substr(start, end - start));
      size_t      vs = end + 1;
      while (vs < line.size() && std::isspace((unsigned char)line[vs]))
        ++vs;
      size_t ve = find_char_or_comment(line, vs, '\0');
      std::string value = rstrip(line.substr(vs, ve - vs));
      prev_name = name.substr(0, 49);
      ini.values[lower(section + "." + name)] = value;
    }
    else if (!ini.error_line)
      ini.error_line = lineno;
  }
  return ini;
}

std::string
get_string(const Ini & ini, const char * sec, const char * name, const char * def)
{
  auto it = ini.values.find(lower(std::string(sec) + "." + name));
  return it == ini.values.end() ? std::string(def) : it->second;
}

double
get_float(const Ini & ini, const char * sec, const char * name, float def)
{
  std::string  s = get_string(ini, sec, name, "");
  const char * v = s.c_str();
  char *       end;
  float        f = std::strtof(v, &end);
  return (double)(end > v ? f : def);
}

// ConfigMap::getBool: exact (case-sensitive) words, else the default
bool
get_bool(const Ini & ini, const char * sec, const char * name, bool def)
{
  const std::string s = get_string(ini, sec, name, "");
  if (s == "1" || s == "yes" || s == "true" || s == "on")
    return true;
  if (s == "0" || s == "no" || s == "false" || s == "off")
    return false;
  return def;
}

long
get_integer(const Ini & ini, const char * sec, const char * name, long def)
{
  std::string  s = get_string(ini, sec, name, "");
  const char * v = s.c_str();
  char *       end;
  long         n = std::strtol(v, &end, 0);
  return end > v ? n : def;
}

} // namespace

extern "C" ek_status
ek_params_from_ini(const char * text, size_t len, ek_params * out)
{
  if (!text || !out)
    return ek_internal::fail(EK_ERR_INVALID, "ek_params_from_ini: null argument");
  Ini ini = parse(text, len);
  if (ini.error_line)
    return ek_internal::fail(EK_ERR_PARSE, "ini parse error at line " + std::to_string(ini.error_line));
  ek_params p;
  std::memset(&p, 0, sizeof p);
  std::string name = get_string(ini, "run", "solver_name", "unknown");
  if (name == "Hydro_Muscl_2D")
    p.dim = 2, p.mhd = 0, p.nbvar = 4, p.ghost_width = 2;
  else if (name == "Hydro_Muscl_3D")
    p.dim = 3, p.mhd = 0, p.nbvar = 5, p.ghost_width = 2;
  else if (name == "MHD_Muscl_2D")
    p.dim = 2, p.mhd = 1, p.nbvar = 8, p.ghost_width = 3;
  else if (name == "MHD_Muscl_3D")
    p.dim = 3, p.mhd = 1, p.nbvar = 8, p.ghost_width = 3;
  else
    return ek_internal::fail(EK_ERR_INVALID, "Solver name not valid : " + name);
  std::strncpy(p.solver_name, name.c_str(), sizeof(p.solver_name) - 1);
  std::string prob = get_string(ini, "hydro", "problem", "unknown");
  std::strncpy(p.problem, prob.c_str(), sizeof(p.problem) - 1);

  p.nStepmax = (int)get_integer(ini, "run", "nstepmax", 1000);
  p.tEnd = get_float(ini, "run", "tend", 0.0f);
  p.tCurrent = get_float(ini, "run", "tCurrent", 0.0f);
  p.nOutput = (int)get_integer(ini, "run", "noutput", 100);
  p.nlog = (int)get_integer(ini, "run", "nlog", 10);
  p.nx = (int)get_integer(ini, "mesh", "nx", 1);
  p.ny = (int)get_integer(ini, "mesh", "ny", 1);
  p.nz = (int)get_integer(ini, "mesh", "nz", 1);
  p.xmin = get_float(ini, "mesh", "xmin", 0.0f);
  p.xmax = get_float(ini, "mesh", "xmax", 1.0f);
  p.ymin = get_float(ini, "mesh", "ymin", 0.0f);
  p.ymax = get_float(ini, "mesh", "ymax", 1.0f);
  p.zmin = get_float(ini, "mesh", "zmin", 0.0f);
  p.zmax = get_float(ini, "mesh", "zmax", 1.0f);
  const char * faces[6] = { "xmin", "xmax", "ymin", "ymax", "zmin", "zmax" };
  for (int f = 0; f < 6; ++f)
    p.bc[f] = (int)get_integer(ini, "mesh", (std::string("boundary_type_") + faces[f]).c_str(), 1);

  std::string rs = get_string(ini, "hydro", "riemann", "approx");
  p.riemann = rs == "llf" ? 1 : rs == "hll" ? 2 : rs == "hllc" ? 3 : rs == "hlld" ? 4 : 0;
  int iv = (int)get_float(ini, "OTHER", "implementationVersion", 0.0f);
  p.implementation_version = (iv == 0 || iv == 1 || iv == 2) ? iv : 0;

  p.gamma0 = get_float(ini, "hydro", "gamma0", 1.4f);
  p.cfl = get_float(ini, "hydro", "cfl", 0.5f);
  p.slope_type = get_float(ini, "hydro", "slope_type", 1.0f);
  p.smallc = get_float(ini, "hydro", "smallc", 1e-10f);
  p.smallr = get_float(ini, "hydro", "smallr", 1e-10f);
  p.cIso = 0.0;
  p.Omega0 = 0.0;

  // HydroParams::init
  p.isize = p.nx + 2 * p.ghost_width;
  p.jsize = p.ny + 2 * p.ghost_width;
  p.ksize = p.nz + 2 * p.ghost_width;
  p.dx = (p.xmax - p.xmin) / p.nx;
  p.dy = (p.ymax - p.ymin) / p.ny;
  p.dz = (p.zmax - p.zmin) / p.nz;
  p.smallp = p.smallc * p.smallc / p.gamma0;
  p.smallpp = p.smallr * p.smallp;
  p.gamma6 = (p.gamma0 + 1.0) / (2.0 * p.gamma0);

  // [output]: IO_ReadWrite.cpp:31-43 (getBool: ConfigMap.cpp:64-82), IO_VTK.cpp:62-66
  std::string odir = get_string(ini, "output", "outputDir", "./");
  std::string opre = get_string(ini, "output", "outputPrefix", "output");
  std::strncpy(p.output_dir, odir.c_str(), sizeof(p.output_dir) - 1);
  std::strncpy(p.output_prefix, opre.c_str(), sizeof(p.output_prefix) - 1);
  p.vtk_enabled = get_bool(ini, "output", "vtk_enabled", true) ? 1 : 0;
  p.vtk_ascii = get_bool(ini, "output", "outputVtkAscii", false) ? 1 : 0;

  // [gravity]: GravityParams (GravityParams.h:32-37), SolverBase.cpp:38; the
  // field is the Rayleigh-Taylor init's uniform one
  // (RayleighTaylorInstabilityParams.h:28-34), zero for the other problems
  p.gravity_enabled = get_bool(ini, "gravity", "enabled", false) ? 1 : 0;
  p.gravity_static = get_bool(ini, "gravity", "static", false) ? 1 : 0;
  p.gravity_hancock = get_bool(ini, "gravity", "hancock_predictor_enabled", false) ? 1 : 0;
  p.gravity_well_balanced = get_bool(ini, "gravity", "well_balanced_reconstruction_enabled", false) ? 1 : 0;
  if (prob == "rayleigh_taylor")
  {
    p.gravity[0] = get_float(ini, "rayleigh_taylor", "gx", 0.0f);
    p.gravity[1] = get_float(ini, "rayleigh_taylor", "gy", -0.1f);
    p.gravity[2] = p.dim == 3 ? get_float(ini, "rayleigh_taylor", "gz", 0.0f) : 0.0;
  }

  // additions of this library, in a section the reference does not read
  std::string prec = lower(get_string(ini, "gb300", "precision", "fp64"));
  p.precision = (prec == "mixed" || prec == "fp32") ? EK_PREC_MIXED : EK_PREC_FP64;
  p.exact_fp = (int)get_integer(ini, "gb300", "exact", 0);
  p.kchunk = (int)get_integer(ini, "gb300", "kchunk", 0);
  p.mhd_stage = (int)get_integer(ini, "gb300", "mhd_stage", 0);
  p.no_tma = get_integer(ini, "gb300", "tma", 1) == 0 ? 1 : 0;
  *out = p;
  return EK_OK;
}
