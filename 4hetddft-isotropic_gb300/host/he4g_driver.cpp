// he4g_driver — a native stand-in for the reference's main program
// (DFT4He3d.f90) on top of the C ABI of include/he4g.h. It reads the same
// namelist input (&input group) and initial state file (readenc modes 0 and
// 2), runs the time loop of DFT4He3d.f90:832-1000 through he4g_step, and
// writes the reference's outputs:
//  - rimp.out / vimp.out / aimp.out: a header line, the initial state at
//    time0, then one line per step at time0 + iteraux*deltatps, format
//    (1x,1p,E15.6,3E18.10), velocities in A/ps and accelerations in A/ps^2
//    (DFT4He3d.f90:804-863);
//  - on stdout, per predictor-corrector step the errHe/errimp line, and every
//    pener steps the particle number, the energy blocks of formats 7010 and
//    7015 and <Lx,Ly,Lz> (DFT4He3d.f90:844-926, 1128-1140);
//  - every pcurr steps density.NNNN.dat in the printoutc layout
//    (printoutc.f90:52-77; DFT4He3d.f90:972-994), psi read back with
//    he4g_get_psi_async so that the copy overlaps the next steps;
//  - with lsurf, the TiO2 surface potential (lsurf3D, Zsurf;
//    DFT4He3d.f90:760-784) in the energy blocks, and uext.dat (:785-792);
//  - DFT4He3d.namelist.read, the echo of the &input group (:195-196), from
//    which the Fortran wrappers read their loop cadence;
//  - timec.dat, the absorber's real part in the y = 0 plane (:704-711);
//  - the hedenini-*.dat and uimp-*.dat cuts through the box centre of the
//    initial density and of uimp after the first evaluation (respar.f90,
//    :391, :649).
//
//   he4g_driver input.nml [--precision fp64|mixed|df64] [--parse]
//
// --parse prints the parsed run as one line of key=value pairs and exits
// without touching a GPU.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "he4g.h"

namespace {

constexpr double kPsToK = 7.63822291;  // DFT4He3d.f90:238, 302

[[noreturn]] void die(const std::string& m) {
  std::fprintf(stderr, "he4g_driver: %s\n", m.c_str());
  std::exit(2);
}

std::string lower(std::string s) {
  for (char& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

// ---------------------------------------------------------------- namelist
// The &input group: name = value pairs separated by commas, blanks or line
// ends, '!' comments, up to the closing '/'. Values are Fortran literals:
// numbers (D or E exponents), logicals (.true., T, .false., F) and quoted
// strings. Keys are case-insensitive.
std::map<std::string, std::string> read_namelist(const std::string& path, const std::string& group) {
  std::ifstream f(path);
  if (!f) die("cannot open " + path);
  std::string text, line;
  while (std::getline(f, line)) {
    bool inq = false;
    char q = 0;
    for (size_t i = 0; i < line.size(); ++i) {  // drop comments outside quotes
      const char c = line[i];
      if (inq) {
        if (c == q) inq = false;
      } else if (c == '\'' || c == '"') {
        inq = true;
        q = c;
      } else if (c == '!') {
        line.resize(i);
        break;
      }
    }
    text += line + "\n";
  }
  const std::string low = lower(text);
  const size_t g = low.find("&" + lower(group));
  if (g == std::string::npos) die("no &" + group + " group in " + path);
  size_t i = g + group.size() + 1;
  std::map<std::string, std::string> out;
  auto skip = [&] {
    while (i < text.size() && (std::isspace(static_cast<unsigned char>(text[i])) || text[i] == ',')) ++i;
  };
  while (true) {
    skip();
    if (i >= text.size() || text[i] == '/' || text[i] == '&') break;
    size_t k = i;
    while (i < text.size() && text[i] != '=' && text[i] != ',' && text[i] != '/' &&
           !std::isspace(static_cast<unsigned char>(text[i])))
      ++i;
    const std::string key = lower(text.substr(k, i - k));
    skip();
    if (i >= text.size() || text[i] != '=') continue;  // a further value of an array item: ignored
    ++i;
    skip();
    std::string val;
    if (text[i] == '\'' || text[i] == '"') {
      const char q = text[i++];
      const size_t e = text.find(q, i);
      if (e == std::string::npos) die("namelist: unterminated string for " + key);
      val = text.substr(i, e - i);
      i = e + 1;
    } else {
      k = i;
      while (i < text.size() && text[i] != ',' && text[i] != '/' && !std::isspace(static_cast<unsigned char>(text[i])))
        ++i;
      val = text.substr(k, i - k);
    }
    out[key] = val;
  }
  return out;
}

double fnum(std::string v) {
  for (char& c : v)
    if (c == 'd' || c == 'D') c = 'e';
  char* end = nullptr;
  const double x = std::strtod(v.c_str(), &end);
  if (end == v.c_str()) die("not a number: " + v);
  return x;
}
bool flog(const std::string& v) {
  const std::string l = lower(v);
  return l == ".true." || l == "t" || l == ".t." || l == "true";
}

// ------------------------------------------------------- list-directed data
// The values of a readenc record stream: blanks/commas separate items,
// "(re,im)" is a complex item, "r*v" repeats v r times.
struct Tokens {
  std::istream& in;
  std::vector<std::string> buf;
  size_t pos = 0;
  explicit Tokens(std::istream& s) : in(s) {}
  bool refill() {
    std::string line;
    while (std::getline(in, line)) {
      buf.clear();
      pos = 0;
      size_t i = 0;
      while (i < line.size()) {
        const char c = line[i];
        if (std::isspace(static_cast<unsigned char>(c)) || c == ',') {
          ++i;
          continue;
        }
        // an item ends at a blank or comma outside parentheses ("(re,im)",
        // "3*(re,im)")
        const size_t k = i;
        bool paren = false;
        while (i < line.size()) {
          const char ch = line[i];
          if (ch == '(') paren = true;
          else if (ch == ')') paren = false;
          else if (!paren && (std::isspace(static_cast<unsigned char>(ch)) || ch == ',')) break;
          ++i;
        }
        buf.push_back(line.substr(k, i - k));
      }
      if (!buf.empty()) return true;
    }
    return false;
  }
  std::string next() {
    if (pos >= buf.size() && !refill()) die("initial state file ends early");
    return buf[pos++];
  }
  void end_record() { pos = buf.size(); }
};

// -------------------------------------------------------------- formatting
std::string fe(double v, int w, int d) {  // Fortran 1P,Ew.d
  char b[64];
  std::snprintf(b, sizeof b, "%*.*E", w, d, v);
  return b;
}
std::string ff(double v, int w, int d) {  // Fortran 0P,Fw.d
  char b[64];
  std::snprintf(b, sizeof b, "%*.*f", w, d, v);
  return b;
}

void check(int rc, const char* what, he4g_run* run) {
  if (rc == 0) return;
  const char* m = run ? he4g_last_error(run) : nullptr;
  die(std::string(what) + " failed (" + std::to_string(rc) + ")" + (m && *m ? std::string(": ") + m : ""));
}

void write_density(const std::string& path, const std::vector<double>& psi, const he4g_config& c, const double r[3],
                   const double v[3], long long iter, double dtps, double time, const std::string& selec,
                   double r_cutoff, double umax, const he4g_obs& o, const he4g_energies& e) {
  std::FILE* f = std::fopen(path.c_str(), "w");
  if (!f) die("cannot write " + path);
  auto f3 = [&](const double* x) {
    std::string s;
    for (int k = 0; k < 3; ++k) s += fe(x[k], 16, 8);
    return s;
  };
  std::fprintf(f, "#  \n#  Density after %15lld iterations\n", iter);
  std::fprintf(f, "#  Actual deltatps....:%20.10E\n#  Total evolution time(ps)...:%20.12E\n", dtps, time);
  std::fprintf(f, "#  Impurity potential.........:  %s\n", selec.c_str());
  std::fprintf(f, "#  r_cutoff_gs:%16.8E\n#  umax_gs....:%16.8E\n", r_cutoff, umax);
  std::fprintf(f, "#  xcm,ycm,zcm:%s\n#  NParticles.:%16.8E\n", f3(o.cm).c_str(), o.npart);
  const std::pair<const char*, double> rows[] = {{"Ekin.......", e.ekin4}, {"Elj........", e.elj4},
                                                 {"Ealphas....", e.ealphas}, {"Ecorr......", e.ecor4},
                                                 {"Esolid.....", e.esolid}, {"Ekinx......", e.ekinx},
                                                 {"Eimpu......", e.eimpu}, {"Etot.......", e.etot}};
  for (const auto& rw : rows) std::fprintf(f, "#  %s:%16.8E\n", rw.first, rw.second);
  std::fprintf(f, "#  <Lx,y,z>...:%s\n#  <x2,y2,z2>.:%s\n#  \n", f3(o.ang).c_str(), f3(o.r2).c_str());
  const double hx = 2 * c.xmax / c.nx, hy = 2 * c.ymax / c.ny, hz = 2 * c.zmax / c.nz;
  std::fprintf(f, "%.17E %.17E %.17E %.17E %.17E %.17E %d %d %d\n", c.xmax, c.ymax, c.zmax, hx, hy, hz, c.nx, c.ny,
               c.nz);
  std::fprintf(f, "%.17E %.17E %.17E\n%.17E %.17E %.17E\n", r[0], r[1], r[2], v[0], v[1], v[2]);
  const size_t n = psi.size() / 2;
  for (size_t p = 0; p < n; ++p)
    std::fprintf(f, "(%.17E,%.17E)%s", psi[2 * p], psi[2 * p + 1], (p % 4 == 3 || p + 1 == n) ? "\n" : " ");
  std::fclose(f);
}

// DFT4He3d.namelist.read: the &input group as read (DFT4He3d.f90:195-196),
// one NAME=value per line; literals as given, strings quoted
void write_namelist_echo(const std::map<std::string, std::string>& nl) {
  std::FILE* f = std::fopen("DFT4He3d.namelist.read", "w");
  if (!f) die("cannot write DFT4He3d.namelist.read");
  std::fprintf(f, "&INPUT\n");
  for (const auto& kv : nl) {
    std::string key = kv.first;
    for (char& c : key) c = static_cast<char>(std::toupper(static_cast<unsigned char>(c)));
    std::string v = kv.second, e = v;
    for (char& c : e)
      if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    std::strtod(e.c_str(), &end);
    const std::string l = lower(v);
    const bool literal = (!e.empty() && end == e.c_str() + e.size()) || l == ".true." || l == ".false." ||
                         l == "t" || l == "f" || l == ".t." || l == ".f.";
    std::fprintf(f, " %s=%s%s%s,\n", key.c_str(), literal ? "" : "'", v.c_str(), literal ? "" : "'");
  }
  std::fprintf(f, " /\n");
  std::fclose(f);
}

// respar.f90: fun(x, y = 0, z = 0), fun(0, y, 0) and fun(0, 0, z) at the box
// centre (ix = nx/2+1 etc.) into name-x/y/z.dat, format (1x,1P,2E14.5), with
// values below 1e-40 in magnitude written as 0
void write_cuts(const std::string& name, const std::vector<double>& fun, const he4g_config& c) {
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const double h[3] = {2 * c.xmax / nx, 2 * c.ymax / ny, 2 * c.zmax / nz};
  const double lo[3] = {-c.xmax, -c.ymax, -c.zmax};
  const int n[3] = {nx, ny, nz};
  const char* ax = "xyz";
  for (int a = 0; a < 3; ++a) {
    const std::string path = name + "-" + ax[a] + ".dat";
    std::FILE* f = std::fopen(path.c_str(), "w");
    if (!f) die("cannot write " + path);
    for (int t = 0; t < n[a]; ++t) {
      const int i = a == 0 ? t : nx / 2, j = a == 1 ? t : ny / 2, k = a == 2 ? t : nz / 2;
      double v = fun[(static_cast<size_t>(k) * ny + j) * nx + i];
      if (std::fabs(v) < 1e-40) v = 0.0;
      std::fprintf(f, " %s%s\n", fe(lo[a] + h[a] * t, 14, 5).c_str(), fe(v, 14, 5).c_str());
    }
    std::fclose(f);
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) die("usage: he4g_driver input.nml [--precision fp64|mixed|df64] [--parse]");
  std::string path = argv[1], prec = "fp64";
  bool parse_only = false;
  for (int a = 2; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--parse")) parse_only = true;
    else if (!std::strcmp(argv[a], "--precision") && a + 1 < argc) prec = argv[++a];
    else die(std::string("unknown option ") + argv[a]);
  }
  const auto nl = read_namelist(path, "input");
  auto has = [&](const char* k) { return nl.count(k) > 0; };
  auto num = [&](const char* k, double d) { return has(k) ? fnum(nl.at(k)) : d; };
  auto str = [&](const char* k, const char* d) { return has(k) ? nl.at(k) : std::string(d); };

  // grid (the reference takes it from the namelist; DFT4He3d.f90:149-168)
  const int nx = static_cast<int>(num("nx", 0)), ny = static_cast<int>(num("ny", nx)),
            nz = static_cast<int>(num("nz", nx));
  const double xmax = num("xmax", 0), ymax = num("ymax", xmax), zmax = num("zmax", xmax);
  if (nx <= 0 || !(xmax > 0)) die("the namelist needs nx and xmax");
  he4g_config c;
  he4g_default_config(&c, nx, ny, nz, xmax, ymax, zmax);
  struct {
    const char* key;
    double* field;
  } reals[] = {{"cp4", &c.cp4},       {"cpp4", &c.cpp4},     {"h2o2m4", &c.h2o2m4}, {"alphas", &c.alphas},
               {"l", &c.l_alpha},     {"eps4", &c.eps4},     {"sigma4", &c.sigma4}, {"lambdah", &c.lambdah},
               {"txmean", &c.txmean}, {"txsurf", &c.txsurf}, {"tymean", &c.tymean}, {"tysurf", &c.tysurf},
               {"tzmean", &c.tzmean}, {"tzsurf", &c.tzsurf}, {"mimpur", &c.mimpur}};
  for (auto& rf : reals)
    if (has(rf.key)) *rf.field = fnum(nl.at(rf.key));
  if (has("npd")) c.npd = static_cast<int>(fnum(nl.at("npd")));
  if (has("icon")) c.icon = static_cast<int>(fnum(nl.at("icon")));
  if (has("lsolid")) c.lsolid = flog(nl.at("lsolid")) ? 1 : 0;
  if (has("core4")) c.core = lower(str("core4", "OT")).find("otc") == 0 ? HE4G_CORE_OTC : HE4G_CORE_OT;
  if (has("lrk")) c.lrk = flog(nl.at("lrk")) ? 1 : 0;
  if (!c.lsolid && c.core == HE4G_CORE_OTC) c.hcg = c.h4;  // DFT4He3d.f90:579-590 (h_cg = h4 without lsolid)
  // time step (DFT4He3d.f90:233-249)
  double deltat = num("deltat", 0.0), dtps = num("deltatps", 0.0);
  if (deltat == 0.0) deltat = dtps / kPsToK;
  if (dtps == 0.0) dtps = deltat * kPsToK;
  if (!(deltat > 0)) die("the namelist needs deltat or deltatps");
  c.deltat = deltat;
  c.precision = prec == "mixed" ? HE4G_PREC_MIXED : prec == "df64" ? HE4G_PREC_DF64 : HE4G_PREC_FP64;
  const std::string selec = str("selec", "Xe_He");
  const double r_cutoff = num("r_cutoff", 2.55), umax = num("umax", 2793.9365463);
  const long long niter = static_cast<long long>(num("niter", 0)), iter0 = static_cast<long long>(num("iter0", 0));
  const long long pener = static_cast<long long>(num("pener", 50)), pcurr = static_cast<long long>(num("pcurr", 0));
  const long long icurr = static_cast<long long>(num("icurr", 0));
  const double time0 = num("time0", -1.0), n4 = num("n4", 0.0);
  const int mode = static_cast<int>(num("mode", 0));
  const std::string filein = str("filedenin", "den.dat");
  double rimp[3] = {num("ximp", 0), num("yimp", 0), num("zimp", 0)};
  double vimp[3] = {num("vximp", 0) * kPsToK, num("vyimp", 0) * kPsToK, num("vzimp", 0) * kPsToK};

  if (!parse_only) write_namelist_echo(nl);
  if (parse_only) {
    std::printf("nx=%d ny=%d nz=%d xmax=%.17g ymax=%.17g zmax=%.17g deltat=%.17g deltatps=%.17g niter=%lld "
                "pener=%lld pcurr=%lld mode=%d lsolid=%d core=%d lrk=%d selec=%s r_cutoff=%.17g umax=%.17g "
                "mimpur=%.17g tzmean=%.17g lambdah=%.17g rimp=%.17g,%.17g,%.17g vimp=%.17g,%.17g,%.17g "
                "filedenin=%s\n",
                nx, ny, nz, xmax, ymax, zmax, deltat, dtps, niter, pener, pcurr, mode, c.lsolid, c.core, c.lrk,
                selec.c_str(), r_cutoff, umax, c.mimpur, c.tzmean, c.lambdah, rimp[0], rimp[1], rimp[2], vimp[0],
                vimp[1], vimp[2], filein.c_str());
    return 0;
  }

  // initial state (readenc.f90:82-128, modes 0 and 2)
  const size_t n = static_cast<size_t>(nx) * ny * nz;
  std::vector<double> psi(2 * n);
  {
    std::ifstream f(filein);
    if (!f) die("cannot open " + filein);
    std::string line;
    std::streampos start = f.tellg();
    while (std::getline(f, line) && !line.empty() && line[0] == '#') start = f.tellg();
    f.seekg(start);
    Tokens tk(f);
    double head[6];
    for (double& h : head) h = fnum(tk.next());
    const int fnx = static_cast<int>(fnum(tk.next())), fny = static_cast<int>(fnum(tk.next())),
              fnz = static_cast<int>(fnum(tk.next()));
    if (fnx != nx || fny != ny || fnz != nz) die("the initial state's grid differs from the namelist's");
    if (mode == 0) {
      const bool limp = flog(tk.next());
      double p[3];
      for (double& x : p) x = fnum(tk.next());
      if (limp)
        for (int k = 0; k < 3; ++k) rimp[k] = p[k];
    } else if (mode == 2) {
      tk.end_record();
      for (double& x : rimp) x = fnum(tk.next());
      tk.end_record();
      for (double& x : vimp) x = fnum(tk.next());
    } else {
      die("mode " + std::to_string(mode) + ": this driver reads readenc modes 0 and 2");
    }
    tk.end_record();
    size_t k = 0;
    while (k < n) {
      std::string t = tk.next();
      long long rep = 1;
      const size_t star = t.find('*');
      if (star != std::string::npos) {
        rep = std::atoll(t.substr(0, star).c_str());
        t = t.substr(star + 1);
      }
      double re, im = 0.0;
      if (!t.empty() && t[0] == '(') {
        const size_t comma = t.find(',');
        re = fnum(t.substr(1, comma - 1));
        im = fnum(t.substr(comma + 1, t.size() - comma - 2));
      } else {
        re = std::sqrt(std::max(fnum(t), 0.0));  // a density: psi = sqrt(den) (readenc.f90:96-99)
      }
      for (long long r = 0; r < rep && k < n; ++r, ++k) {
        psi[2 * k] = re;
        psi[2 * k + 1] = im;
      }
    }
  }

  // tables, run, state: the set-up of DFT4He3d.f90:518-644
  std::vector<double> potion(c.npot);
  check(he4g_build_tables(&c, selec.c_str(), r_cutoff, umax, nullptr, nullptr, nullptr, potion.data()),
        "he4g_build_tables", nullptr);
  he4g_run* run = nullptr;
  check(he4g_create(&c, nullptr, nullptr, nullptr, potion.data(), &run), "he4g_create", nullptr);
  {
    // timec.dat (DFT4He3d.f90:704-711): x, z and the absorber's real part at iy = ny/2+1
    std::vector<float> tc(n);
    check(he4g_build_timec(&c, tc.data()), "he4g_build_timec", nullptr);
    std::FILE* f = std::fopen("timec.dat", "w");
    if (!f) die("cannot write timec.dat");
    const double hx = 2 * c.xmax / nx, hz = 2 * c.zmax / nz;
    for (int k = 0; k < nz; ++k) {
      for (int i = 0; i < nx; ++i)
        std::fprintf(f, " %24.16E %24.16E %16.8E\n", -c.xmax + hx * i, -c.zmax + hz * k,
                     static_cast<double>(tc[(static_cast<size_t>(k) * ny + ny / 2) * nx + i]));
      std::fprintf(f, " \n");
    }
    std::fclose(f);
  }
  check(he4g_set_state(run, psi.data(), rimp, vimp), "he4g_set_state", run);
  {
    // the initial density (DFT4He3d.f90:391) and uimp after the first evaluation (:649)
    std::vector<double> field(n);
    check(he4g_get_den(run, field.data()), "he4g_get_den", run);
    write_cuts("hedenini", field, c);
    check(he4g_get_field(run, 3, field.data()), "he4g_get_field", run);
    write_cuts("uimp", field, c);
  }
  // the TiO2 surface (DFT4He3d.f90:760-784): uext enters the energy only
  if (has("lsurf") && flog(nl.at("lsurf"))) {
    std::vector<double> uext(n);
    const bool l3d = has("lsurf3d") && flog(nl.at("lsurf3d"));
    check(he4g_build_uext(&c, l3d ? 1 : 0, num("zsurf", -25.0), uext.data()), "he4g_build_uext", run);
    check(he4g_set_uext(run, uext.data()), "he4g_set_uext", run);
    // uext.dat (DFT4He3d.f90:785-792): z and uext(3,5,iz)
    std::FILE* f = std::fopen("uext.dat", "w");
    if (!f) die("cannot write uext.dat");
    const double hz = 2 * c.zmax / nz;
    for (int k = 0; k < nz; ++k)
      std::fprintf(f, " %24.16E %24.16E\n", -c.zmax + hz * k, uext[(static_cast<size_t>(k) * ny + 4) * nx + 2]);
    std::fclose(f);
  }

  std::FILE* fo[3] = {std::fopen(str("filerimp", "rimp.out").c_str(), "w"),
                      std::fopen(str("filevimp", "vimp.out").c_str(), "w"),
                      std::fopen(str("fileaimp", "aimp.out").c_str(), "w")};
  if (!fo[0] || !fo[1] || !fo[2]) die("cannot open the trajectory files");
  std::fprintf(fo[0], "# Tiempo(ps), x(AA), y(AA), z(AA)\n");
  std::fprintf(fo[1], "# Tiempo(ps), Vx(AA/ps), Vy(AA/ps), Vz(AA/ps)\n");
  std::fprintf(fo[2], "# Tiempo(ps), Ax(AA/ps**2), Ay(AA/ps**2), Az(AA/ps**2)\n");
  auto traj = [&](double t) {
    double r[3], v[3], a[3];
    check(he4g_get_impurity(run, r, v, a), "he4g_get_impurity", run);
    const double vs = 1.0 / kPsToK, as = vs * vs;
    std::fprintf(fo[0], " %s%s%s%s\n", fe(t, 15, 6).c_str(), fe(r[0], 18, 10).c_str(), fe(r[1], 18, 10).c_str(),
                 fe(r[2], 18, 10).c_str());
    std::fprintf(fo[1], " %s%s%s%s\n", fe(t, 15, 6).c_str(), fe(v[0] * vs, 18, 10).c_str(),
                 fe(v[1] * vs, 18, 10).c_str(), fe(v[2] * vs, 18, 10).c_str());
    std::fprintf(fo[2], " %s%s%s%s\n", fe(t, 15, 6).c_str(), fe(a[0] * as, 18, 10).c_str(),
                 fe(a[1] * as, 18, 10).c_str(), fe(a[2] * as, 18, 10).c_str());
    for (std::FILE* f : fo) std::fflush(f);
  };
  traj(time0);

  double eold = 0.0;
  std::vector<double> dump(2 * n);
  bool dump_pending = false;
  for (long long iter = iter0 + 1; iter <= niter; ++iter) {
    const long long iteraux = iter - iter0;
    double errHe = 0.0, errimp = 0.0;
    check(he4g_step(run, 1, &errHe, &errimp), "he4g_step", run);
    if (!(iteraux <= 3 || c.lrk)) std::printf(" Error( He, imp) (From Steppc)...%s%s\n", fe(errHe, 15, 6).c_str(),
                                              fe(errimp, 15, 6).c_str());
    const double t = time0 + iteraux * dtps;
    traj(t);
    he4g_energies e{};
    he4g_obs o{};
    const bool print_e = pener > 0 && iter % pener == 0;
    const bool write_d = pcurr > 0 && iteraux % pcurr == 0;
    if (print_e || write_d) {
      check(he4g_energy(run, &e), "he4g_energy", run);
      check(he4g_observables(run, n4, &o), "he4g_observables", run);
    }
    if (print_e) {
      std::printf(" Iteration....:%10lld\n", iter);
      std::printf(" Number of particles....:%s\n", fe(o.npart, 18, 10).c_str());
      std::printf("\n\n    ITERATIVE PROCEDURE \n\n");
      std::printf("    Total Energy (He).......... %s K +- %s K\n", ff(e.etot4, 18, 6).c_str(),
                  fe(e.etot4 - eold, 12, 4).c_str());
      std::printf("    Energy per particle (He)... %s K\n\n", ff(n4 != 0 ? e.etot4 / n4 : 0.0, 18, 6).c_str());
      std::printf("    Kinetic Energy (He)........ %s K\n", ff(e.ekin4, 18, 6).c_str());
      std::printf("    Lennard-Jones Energy (He).. %s K\n", ff(e.elj4, 18, 6).c_str());
      std::printf("    Alpha_s term  energy (He).. %s K\n", ff(e.ealphas, 18, 6).c_str());
      std::printf("    Solid energy (He) ......... %s K\n", ff(e.esolid, 18, 6).c_str());
      std::printf("    Correlation Energy  (He)... %s K\n", ff(e.ecor4, 18, 6).c_str());
      std::printf("    Impurity energy (X->He) ... %s K\n", ff(e.eimpu, 18, 6).c_str());
      std::printf("    Kinetic energy (X) ........ %s K\n", ff(e.ekinx, 18, 6).c_str());
      std::printf("    Interaction energy (X-He) . %s K\n", ff(e.eHeX, 18, 6).c_str());
      std::printf("    Spin-Orbit energy (X) ..... %s K\n", ff(0.0, 18, 6).c_str());
      std::printf("    TOTAL energy (He+X) ....... %s K\n \n", ff(e.etot, 18, 6).c_str());
      std::printf("<Lx,Ly,Lz>.......:%s%s%s\n", fe(o.ang[0], 20, 11).c_str(), fe(o.ang[1], 20, 11).c_str(),
                  fe(o.ang[2], 20, 11).c_str());
      std::fflush(stdout);
      eold = e.etot4;
    }
    if (write_d) {
      // the previous dump's copy has landed before its buffer is reused
      if (dump_pending) check(he4g_wait_psi(run), "he4g_wait_psi", run);
      check(he4g_get_psi_async(run, dump.data()), "he4g_get_psi_async", run);
      check(he4g_wait_psi(run), "he4g_wait_psi", run);
      dump_pending = false;
      double r[3], v[3], a[3];
      check(he4g_get_impurity(run, r, v, a), "he4g_get_impurity", run);
      char name[64];
      std::snprintf(name, sizeof name, "density.%04lld.dat", iteraux / pcurr + icurr);
      write_density(name, dump, c, r, v, iter, dtps, t, selec, r_cutoff, umax, o, e);
    }
  }
  for (std::FILE* f : fo) std::fclose(f);
  he4g_destroy(run);
  return 0;
}
