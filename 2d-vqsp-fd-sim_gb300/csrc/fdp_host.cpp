// fdp_host: a drop-in driver for reference job directories.
//
// Reads the reference's input files, performs its set-up in main.F90's
// order (READ_OPEN, AUX1, READ_MODEL, READ_MODEL_PAR, OPEN_SR_FILE,
// PRE_NR_COEF1, PPML; main.F90:60-82), runs the time loop on the GPU through
// include/fdp.h, and writes the reference's output files:
//   REC_UW_<j>.asc, REC_Q_<j>.asc     store_seismograms.F90:140-154
//   REC_STRESS_<j>.asc                store_seismograms_pressure.F90:76-83
//   SNAP.V<it>, SNAP.Q<it>            store_snapshots.F90:173-190
// It stands in for the Fortran driver where no Fortran compiler exists.
//
// usage: fdp_host [--dir DIR] [--precision f32|f64] [--device N]
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "fdp.h"
#include "fdp_io.h"
#include "fdp_prep.h"

namespace {

struct Opts {
  std::string dir = ".";
  int prec = FDP_F32;
  int device = 0;
};

[[noreturn]] void die(const std::string& msg, FILE* log) {
  std::fprintf(stderr, "fdp_host: %s\n", msg.c_str());
  if (log) { std::fprintf(log, " %s\n", msg.c_str()); std::fclose(log); }
  std::exit(1);
}

std::string slurp(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return "";
  std::stringstream s;
  s << f.rdbuf();
  return s.str();
}

bool exists(const std::string& path) { return (bool)std::ifstream(path); }

// namelist value or empty string
std::string nml(const std::string& text, const char* group, const char* name) {
  char buf[512];
  if (fdp_io_namelist_get(text.c_str(), group, name, buf, sizeof buf) != FDP_OK) return "";
  return buf;
}

double to_real(const std::string& v) {
  std::string s = v;
  for (char& c : s) if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(s.c_str(), nullptr);
}

bool to_logical(const std::string& v) {
  std::string s;
  for (char c : v) if (c != '.') s += (char)std::toupper((unsigned char)c);
  return !s.empty() && s[0] == 'T';
}

std::string trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

// Fortran NINT: round half away from zero
int nint(double x) { return (int)(x >= 0 ? std::floor(x + 0.5) : -std::floor(-x + 0.5)); }

std::string efmt(double v) {
  char b[32];
  fdp_io_format_e(v, 13, 6, b);
  return std::string(" ") + b;
}

template <class T> int run(const Opts& o) {
  const std::string D = o.dir + "/";
  // main.F90:52-54
  std::string job;
  {
    std::ifstream f(D + "HF_2DFD_VS_PORO");
    if (!f || !std::getline(f, job)) die("HF_2DFD_VS_PORO not found", nullptr);
    job = trim(job);
  }
  FILE* log = std::fopen((D + job + ".LOG").c_str(), "w");
  if (log) std::fprintf(log, " LOG_FILE: JOB_NAME =%s\n", job.c_str());
  // read_open.F90:83-95
  if (!exists(D + job + ".IN")) die(job + ".IN NOT FOUND", log);
  const std::string IN = slurp(D + job + ".IN"), INM = slurp(D + job + ".INM");
  if (INM.empty()) die(job + ".INM NOT FOUND", log);
  auto get = [&](const std::string& text, const char* g, const char* n, const std::string& dflt) {
    const std::string v = nml(text, g, n);
    return v.empty() ? dflt : v;
  };
  // CONTROLDATA (read_open.F90:107-113)
  const int TPML = std::atoi(get(IN, "CONTROLDATA", "TPML", "0").c_str());
  const bool SI = to_logical(get(IN, "CONTROLDATA", "STRESS_IMAGING", "T"));
  // NAMES (read_open.F90:102-116)
  const std::string MO = trim(get(INM, "NAMES", "MO_FILE_NAME", job + ".MO"));
  const std::string JMH = trim(get(INM, "NAMES", "JMH_FILE_NAME", job + ".JMH"));
  // CONTROLDATA1 (read_open.F90:118-128); default-real literals
  const std::string mt_s = nml(IN, "CONTROLDATA1", "MT");
  if (mt_s.empty()) die("CONTROLDATA1 lacks MT", log);
  const float MT = (float)to_real(mt_s);
  const T R = (T)to_real(get(IN, "CONTROLDATA1", "R", std::to_string((double)0.001f)));
  const T TAU = (T)to_real(get(IN, "CONTROLDATA1", "TAU", "1.5"));
  const T POW = (T)to_real(get(IN, "CONTROLDATA1", "POW", "2"));
  const T SF = (T)to_real(get(IN, "CONTROLDATA1", "SF", "0"));
  const T WC = (T)to_real(get(IN, "CONTROLDATA1", "WC", "0"));
  const int IPAS2 = std::atoi(get(IN, "CONTROLDATA1", "IPAS2", "1000").c_str());
  // NAMES_SR_REC, KEYS
  const std::string SRF = trim(get(IN, "NAMES_SR_REC", "SR_FILE_NAME", "STF.DAT"));
  const std::string RECF = trim(get(IN, "NAMES_SR_REC", "REC_FILE_NAME", "REC.DAT"));
  const bool TLV = to_logical(get(IN, "KEYS", "KEY_TLV", "T"));
  const bool SNV = to_logical(get(IN, "KEYS", "KEY_SNV", "F"));
  const bool TLQ = to_logical(get(IN, "KEYS", "KEY_TLQ", "F"));
  const bool TLP = to_logical(get(IN, "KEYS", "KEY_TLP", "F"));
  if (!(TLV || SNV)) die("NONE OF TL_ AND SN_ OUTPUT FILES IS REQUIRED", log);  // read_open.F90:139-142
  // CONTROLDATA2 (read_open.F90:144-153)
  const int MX = std::atoi(nml(INM, "CONTROLDATA2", "MX").c_str());
  int MZ = std::atoi(nml(INM, "CONTROLDATA2", "MZ").c_str());
  const T H = (T)to_real(nml(INM, "CONTROLDATA2", "H"));
  const T DT = (T)to_real(nml(INM, "CONTROLDATA2", "DT_VS"));
  const float XBMIN = (float)to_real(get(INM, "CONTROLDATA2", "XBMIN", "0"));
  if (MX <= 0 || MZ <= 0 || !(H > 0) || !(DT > 0)) die("CONTROLDATA2 incomplete", log);
  if (SI) MZ += 2;
  const int MT2 = (int)((T)MT / DT) + 1;
  // SOURCE (read_open.F90:161-169)
  float XS = std::fabs((float)to_real(get(IN, "SOURCE", "X_SOURCE", "0")));
  float ZS = std::fabs((float)to_real(get(IN, "SOURCE", "Z_SOURCE", "0")));
  const int KEY_SOUR = std::atoi(get(IN, "SOURCE", "KEY_SOUR", "0").c_str());
  const T QR = (T)to_real(get(IN, "SOURCE", "QR", "0"));
  if (SI) ZS = (float)((T)ZS + (T)2 * H);
  const int LIN_X = nint((double)((T)(XS - XBMIN) / H));
  const int LIN_Z = nint((double)((T)ZS / H));
  // NONREF (read_open.F90:174-188)
  const T WB = (T)to_real(get(IN, "NONREF", "WB", "0.4"));
  const int KTBO = std::atoi(get(IN, "NONREF", "KTBO", "0").c_str());
  const T THPP = (T)to_real(get(IN, "NONREF", "THPPBO", "0.19757"));
  const T THSS = (T)to_real(get(IN, "NONREF", "THSSBO", "0.70511"));
  const T OMG = (T)to_real(get(IN, "NONREF", "OMG", "0")) / (T)6.283185307179586476925286766559;
  // REC (read_open.F90:213-240)
  std::vector<int32_t> IRX, LRX, IRZ, LRZ;
  int MR = 0;
  if (TLV) {
    MR = std::atoi(get(IN, "REC", "MR", "0").c_str());
    std::ifstream f(D + RECF);
    if (!f) die(RECF + " NOT FOUND", log);
    for (int j = 0; j < MR; ++j) {
      std::string name;
      int a, b, c, d;
      if (!(f >> name >> a >> b >> c >> d)) die("REC.DAT has fewer than MR receivers", log);
      IRX.push_back(a); LRX.push_back(b); IRZ.push_back(c); LRZ.push_back(d);
    }
  }
  // AUX1
  const int PMLL = 1 - TPML, PMLXH = MX + TPML, PMLZH = MZ + TPML;
  const int NX = PMLXH - PMLL + 1, NZ = PMLZH + 1;
  // READ_MODEL (read_model.F90:57-89)
  if (!exists(D + JMH)) die(JMH + " NOT FOUND", log);
  if (!exists(D + MO)) die(MO + " NOT FOUND", log);
  const int nrows = SI ? MZ - 1 : MZ + 1;
  std::vector<int32_t> rows((size_t)nrows * MX), jm((size_t)NX * NZ);
  for (int r = 0; r < nrows; ++r) {
    int64_t nb = 0;
    if (fdp_io_read_record((D + JMH).c_str(), r, &rows[(size_t)r * MX], (int64_t)MX * 4, &nb) != FDP_OK ||
        nb != (int64_t)MX * 4)
      die("bad JM record " + std::to_string(r + 1) + " in " + JMH, log);
  }
  if (fdp_prep_expand_jm(MX, MZ, TPML, SI, rows.data(), jm.data()) != FDP_OK) die("READ_MODEL failed", log);
  // READ_MODEL_PAR (read_model_par.F90:37-74)
  int32_t jmnumr = 0;
  int64_t nb = 0;
  if (fdp_io_read_record((D + MO).c_str(), 0, &jmnumr, 4, &nb) != FDP_OK) die("bad JMNUM record in " + MO, log);
  const int JMNUM = std::abs(jmnumr);
  std::vector<T> table((size_t)JMNUM * 24);
  if (fdp_io_read_record((D + MO).c_str(), 1, table.data(), (int64_t)table.size() * sizeof(T), &nb) != FDP_OK ||
      nb != (int64_t)table.size() * (int64_t)sizeof(T))
    die("bad material record in " + MO + " (precision mismatch?)", log);
  fdp_prep_scale_table(o.prec, JMNUM, (double)DT, (double)H, table.data());
  // OPEN_SR_FILE (open_sr_file.F90:61-110)
  std::vector<T> st, sv;
  {
    std::ifstream f(D + SRF);
    if (!f) die(SRF + " NOT FOUND", log);
    std::string a, b;
    while (f >> a >> b) { st.push_back((T)to_real(a)); sv.push_back((T)to_real(b)); }
  }
  std::vector<T> sourtf((size_t)2 * MT2);
  if (fdp_prep_source(o.prec, (int)st.size(), st.data(), sv.data(), MT2, (double)DT, (double)H, KEY_SOUR, (double)QR,
                      sourtf.data()) != FDP_OK)
    die("OPEN_SR_FILE failed", log);
  // PRE_NR_COEF1 and PPML
  std::vector<T> ab(16);
  if (fdp_prep_bottom_nr(o.prec, MX, MZ, TPML, KTBO, (double)DT, (double)H, (double)OMG, (double)WB, (double)THPP,
                         (double)THSS, jm.data(), JMNUM, table.data(), ab.data()) != FDP_OK)
    die("PRE_NR_COEF1 failed", log);
  std::vector<std::vector<T>> prof(24);
  std::vector<void*> pp(24);
  for (int k = 0; k < 24; ++k) {
    const bool z = (k >= 8 && k < 12) || k >= 20;
    const int nj = (k < 12) ? TPML + 1 : TPML + 2;
    prof[k].resize((size_t)nj * (z ? NX : NZ));
    pp[k] = prof[k].data();
  }
  if (fdp_prep_pml(o.prec, MX, MZ, TPML, KTBO, (double)R, (double)TAU, (double)POW, (double)SF, (double)WC, (double)DT,
                   (double)H, jm.data(), JMNUM, table.data(), pp.data()) != FDP_OK)
    die("PPML failed", log);
  // TIME_LOOP on the GPU
  fdp_grid g{};
  g.mx = MX; g.mz = MZ; g.tpml = TPML; g.stress_imaging = SI; g.lin_x = LIN_X; g.lin_z = LIN_Z;
  g.precision = o.prec; g.device = o.device; g.h = (double)H; g.dt = (double)DT; g.tau_eps = 0.0;
  fdp_ctx* ctx = nullptr;
  auto ck = [&](int rc, const char* what) {
    if (rc != FDP_OK) die(std::string(what) + ": " + fdp_last_error(ctx), log);
  };
  ck(fdp_create(&g, &ctx), "fdp_create");
  ck(fdp_set_medium(ctx, jm.data(), NX, NZ, JMNUM, table.data()), "fdp_set_medium");
  ck(fdp_set_pml(ctx, pp.data()), "fdp_set_pml");
  ck(fdp_set_bottom_nr(ctx, ab.data()), "fdp_set_bottom_nr");
  ck(fdp_set_source(ctx, sourtf.data(), MT2), "fdp_set_source");
  const int flags = (TLV ? FDP_REC_TLV : 0) | (TLQ ? FDP_REC_TLQ : 0) | (TLP ? FDP_REC_TLP : 0);
  ck(fdp_set_receivers(ctx, IRX.data(), LRX.data(), IRZ.data(), LRZ.data(), MR, flags), "fdp_set_receivers");
  const int chunk = 500;
  std::vector<T> rec((size_t)chunk * MR * FDP_REC_VALUES);
  std::vector<T> snap((size_t)2 * NX * NZ);
  std::vector<std::string> uw, qf, sf;
  for (int j = 1; j <= MR; ++j) {
    uw.push_back(D + "REC_UW_" + std::to_string(j) + ".asc");
    qf.push_back(D + "REC_Q_" + std::to_string(j) + ".asc");
    sf.push_back(D + "REC_STRESS_" + std::to_string(j) + ".asc");
  }
  // time_loop.F90:79-86: a file STOP in the job directory ends the run
  // before the next level; the level is written into it, list-directed,
  // and the files of the levels run so far are written.  The reference
  // looks before every level; here the levels of a chunk run in steps of
  // kStep (one captured graph each), the host waiting for each step and
  // looking before the next, so a stop lands at most kStep levels after
  // the file appears (the wait costs the device about 20 us per step).
  const int kStep = 32;
  bool stopped = false;
  for (int it0 = 1; it0 <= MT2 && !stopped;) {
    int it1 = std::min(MT2, it0 + chunk - 1);
    if (SNV) it1 = std::min(it1, (it0 / IPAS2 + 1) * IPAS2);
    int it = it0;
    while (it <= it1) {
      if (exists(D + "STOP")) {
        if (FILE* stf = std::fopen((D + "STOP").c_str(), "w")) {
          std::fprintf(stf, "%12d\n", it);
          std::fclose(stf);
        }
        stopped = true;
        break;
      }
      const int e = std::min(it1, it + kStep - 1);
      ck(fdp_run(ctx, it, e), "fdp_run");
      ck(fdp_synchronize(ctx), "fdp_synchronize");
      it = e + 1;
    }
    if (it == it0) break;
    it1 = it - 1;
    const int n = it1 - it0 + 1;
    if (MR > 0 && (TLV || TLP)) {
      ck(fdp_get_receivers(ctx, it0, n, rec.data()), "fdp_get_receivers");
      for (int j = 0; j < MR; ++j) {
        FILE* fu = TLV ? std::fopen(uw[j].c_str(), "a") : nullptr;
        FILE* fq = (TLV && TLQ) ? std::fopen(qf[j].c_str(), "a") : nullptr;
        FILE* fs = TLP ? std::fopen(sf[j].c_str(), "a") : nullptr;
        for (int k = 0; k < n; ++k) {
          const T* r = &rec[((size_t)k * MR + j) * FDP_REC_VALUES];
          const std::string t = efmt((double)(DT * (T)(it0 + k)));
          if (fu) std::fprintf(fu, "%s%s%s%s%s\n", t.c_str(), efmt(r[0]).c_str(), efmt(r[1]).c_str(),
                               efmt(r[2]).c_str(), efmt(r[3]).c_str());
          if (fq) std::fprintf(fq, "%s%s%s%s%s\n", t.c_str(), efmt(r[4]).c_str(), efmt(r[5]).c_str(),
                               efmt(r[6]).c_str(), efmt(r[7]).c_str());
          if (fs) std::fprintf(fs, "%s%s%s\n", t.c_str(), efmt(r[8]).c_str(), efmt(r[9]).c_str());
        }
        if (fu) std::fclose(fu);
        if (fq) std::fclose(fq);
        if (fs) std::fclose(fs);
      }
    }
    if (SNV && it1 % IPAS2 == 0 && !stopped) {
      char name[32];
      std::snprintf(name, sizeof name, "SNAP.V%06d", it1);
      ck(fdp_get_snapshot(ctx, FDP_SNAP_UM | FDP_SNAP_WM, snap.data()), "fdp_get_snapshot");
      std::remove((D + name).c_str());
      fdp_io_append_record((D + name).c_str(), snap.data(), (int64_t)snap.size() * sizeof(T));
      if (TLQ) {
        std::snprintf(name, sizeof name, "SNAP.Q%06d", it1);
        ck(fdp_get_snapshot(ctx, FDP_SNAP_QX | FDP_SNAP_QZ, snap.data()), "fdp_get_snapshot");
        std::remove((D + name).c_str());
        fdp_io_append_record((D + name).c_str(), snap.data(), (int64_t)snap.size() * sizeof(T));
      }
    }
    if (log) std::fprintf(log, "%6d\n", it1);
    it0 = it1 + 1;
  }
  fdp_destroy(ctx);
  if (log) std::fclose(log);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  Opts o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--dir" && i + 1 < argc) o.dir = argv[++i];
    else if (a == "--precision" && i + 1 < argc) o.prec = std::string(argv[++i]) == "f64" ? FDP_F64 : FDP_F32;
    else if (a == "--device" && i + 1 < argc) o.device = std::atoi(argv[++i]);
    else {
      std::fprintf(stderr, "usage: fdp_host [--dir DIR] [--precision f32|f64] [--device N]\n");
      return 2;
    }
  }
  return o.prec == FDP_F64 ? run<double>(o) : run<float>(o);
}
