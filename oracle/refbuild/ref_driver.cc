// Command-line driver around the UNMODIFIED reference generator sources, used only
// to produce golden vectors for the test suite (test infrastructure, never shipped,
// never on the product path). It is compiled together with the reference's own
// library sources by oracle/refbuild/Makefile; the result lands in oracle/_ref/.
//
// The driver reaches the reference through its public API only:
//   gra::MGraniitti::ReadInput        (src/MGraniitti.cc:318)
//   gra::MProcess::post_Constructor   (src/MContinuum.cc:64)
//   gra::MEikonal::S3Constructor      (src/MEikonal.cc:46)
//   gra::MProcess::EventWeight        (include/Graniitti/MProcess.h:84, src/MContinuum.cc:164)
//   gra::MGraniitti::Initialize/GetXS (src/MGraniitti.cc:1016, include/Graniitti/MGraniitti.h:166)
//
// Modes (all numbers little-endian binary doubles):
//   weights <card> <process> <u.bin> <dim> <out.bin> [options]
//       u.bin holds n*stride doubles, point-major (stride = dim unless --stride);
//       the first dim coordinates are the process's hypercube vector. With
//       --replay SPEC (comma list; 'h' = 0.5, k = coordinate k of the point) the
//       listed values are served, in order, to the draws the process makes from its
//       random-number generator (off-shell masses, decay angles) for that point. out.bin receives, per point,
//       REC doubles: W, kin_ok, fid_ok, veto_ok, amp_ok, t1, t2, m2, then the
//       4-momenta (px,py,pz,E) of pfinal[1], pfinal[2], pfinal[3], pfinal[4].
//   eikonal <card> <process> <out.bin> [options]
//       writes sigma_tot, sigma_el, sigma_inel [barn], then NBT+1 rows of
//       (b, Re, Im) of the density table and NKT2+1 rows of (kt2, Re, Im) of the
//       screening table.
//   vegas <card> <process> [options]   prints "sigma err" [barn].
//
// Options: --nbt N --nkt2 N --loopkt N --loopphi N --maxloopkt X --offshellff K
//          --ncall N --iter N --cores N --precision X --stride S --replay SPEC
//          --leaves N (append the 4-momenta of the first N final-state leaves of the
//          central decay tree to each record)

#include <cstdio>
#include <cstdlib>
#include <functional>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "Graniitti/MContinuum.h"
#include "Graniitti/MGraniitti.h"
#include "Graniitti/MRegge.h"

namespace {

struct Opts {
  int         stride = 0;
  std::string replay;
  int    nbt = 0, nkt2 = 0;
  int    loopkt = -1, loopphi = -1;
  double maxloopkt = -1;
  int    offshellff = -1;
  int    ncall = -1, iter = -1, cores = -1;
  double precision = -1;
  int    leaves = 0;
};

Opts parse_opts(int argc, char **argv, int first) {
  Opts o;
  for (int i = first; i + 1 < argc; i += 2) {
    const std::string k = argv[i];
    const char *      v = argv[i + 1];
    if (k == "--nbt") o.nbt = std::atoi(v);
    else if (k == "--nkt2") o.nkt2 = std::atoi(v);
    else if (k == "--loopkt") o.loopkt = std::atoi(v);
    else if (k == "--loopphi") o.loopphi = std::atoi(v);
    else if (k == "--maxloopkt") o.maxloopkt = std::atof(v);
    else if (k == "--offshellff") o.offshellff = std::atoi(v);
    else if (k == "--ncall") o.ncall = std::atoi(v);
    else if (k == "--iter") o.iter = std::atoi(v);
    else if (k == "--cores") o.cores = std::atoi(v);
    else if (k == "--precision") o.precision = std::atof(v);
    else if (k == "--stride") o.stride = std::atoi(v);
    else if (k == "--replay") o.replay = v;
    else if (k == "--leaves") o.leaves = std::atoi(v);
    else {
      std::fprintf(stderr, "unknown option %s\n", k.c_str());
      std::exit(2);
    }
  }
  return o;
}

void apply_loop_numerics(gra::MProcess *proc, const Opts &o) {
  if (o.loopkt > 0) proc->Eikonal.Numerics.NumberLoopKT = o.loopkt;
  if (o.loopphi > 0) proc->Eikonal.Numerics.NumberLoopPHI = o.loopphi;
  if (o.maxloopkt > 0) proc->Eikonal.Numerics.MaxLoopKT = o.maxloopkt;
}

// The Regge parameter block is read lazily on the first amplitude call; one
// throw-away weight evaluation makes it resident so that the form-factor mode can
// be overridden before any recorded point.
void force_regge_init(gra::MProcess *proc, unsigned dim, const Opts &o) {
  if (o.offshellff < 0) return;
  std::vector<double> u(dim, 0.5);
  gra::AuxIntData     aux;
  proc->EventWeight(u, aux);
  gra::PARAM_REGGE::offshellFF = o.offshellff;
}

std::vector<double> read_doubles(const std::string &fn) {
  std::ifstream f(fn, std::ios::binary | std::ios::ate);
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", fn.c_str());
    std::exit(2);
  }
  const std::streamsize bytes = f.tellg();
  f.seekg(0);
  std::vector<double> v(bytes / sizeof(double));
  f.read(reinterpret_cast<char *>(v.data()), bytes);
  return v;
}

void write_doubles(const std::string &fn, const std::vector<double> &v) {
  std::ofstream f(fn, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(double));
}

void setup(gra::MGraniitti &gen, const std::string &card, const std::string &process,
           const Opts &o) {
  gen.HILJAA = true;
  gen.ReadInput(card, process);
  apply_loop_numerics(gen.proc, o);
  if (o.cores >= 0) gen.SetCores(o.cores);
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: grn_ref weights|eikonal|vegas <card> <process> ...\n");
    return 2;
  }
  const std::string mode    = argv[1];
  const std::string card    = argv[2];
  const std::string process = argv[3];

  try {
    if (mode == "weights") {
      if (argc < 7) return 2;
      const std::string ufile = argv[4];
      const unsigned    dim   = std::atoi(argv[5]);
      const std::string ofile = argv[6];
      const Opts        o     = parse_opts(argc, argv, 7);

      gra::MGraniitti gen;
      setup(gen, card, process, o);
      gra::MProcess *proc = gen.proc;
      proc->post_Constructor();
      if (proc->GetdLIPSDim() != dim) {
        std::fprintf(stderr, "dimension mismatch: process has %u\n", proc->GetdLIPSDim());
        return 3;
      }
      if (proc->GetScreening()) {
        proc->Eikonal.S3Constructor(proc->GetMandelstam_s(), proc->GetInitialState(), false, o.nbt,
                                    o.nkt2);
      }
      force_regge_init(proc, dim, o);

      const std::vector<double> u = read_doubles(ufile);
      const unsigned            stride = o.stride > 0 ? o.stride : dim;
      const std::size_t         n = u.size() / stride;
      std::vector<int>          spec;  // -1 = 0.5, else coordinate index
      for (std::size_t a = 0; a < o.replay.size();) {
        std::size_t b = o.replay.find(',', a);
        if (b == std::string::npos) b = o.replay.size();
        const std::string tok = o.replay.substr(a, b - a);
        spec.push_back(tok == "h" ? -1 : std::atoi(tok.c_str()));
        a = b + 1;
      }
      const int                 REC = 8 + 16 + 4 * o.leaves;
      std::vector<double>       out(n * REC, 0.0);
      std::vector<double>       x(dim);
      for (std::size_t i = 0; i < n; ++i) {
        for (unsigned d = 0; d < dim; ++d) x[d] = u[i * stride + d];
        gra::replay::clear();
        for (int k : spec) gra::replay::push(k < 0 ? 0.5 : u[i * stride + k]);
        gra::AuxIntData aux;
        const double    W = proc->EventWeight(x, aux);
        if (!spec.empty() && gra::replay::remaining() != 0) {
          std::fprintf(stderr, "replay: %zu values not consumed at point %zu\n",
                       gra::replay::remaining(), i);
          return 5;
        }
        double *        r = &out[i * REC];
        r[0]              = W;
        r[1]              = aux.kinematics_ok;
        r[2]              = aux.fidcuts_ok;
        r[3]              = aux.vetocuts_ok;
        r[4]              = aux.amplitude_ok;
        r[5]              = proc->lts.t1;
        r[6]              = proc->lts.t2;
        r[7]              = proc->lts.m2;
        for (int k = 0; k < 4; ++k) {
          const gra::M4Vec &p = proc->lts.pfinal[k + 1];
          r[8 + 4 * k + 0]    = p.Px();
          r[8 + 4 * k + 1]    = p.Py();
          r[8 + 4 * k + 2]    = p.Pz();
          r[8 + 4 * k + 3]    = p.E();
        }
        // final-state leaves of the central decay tree, depth first
        if (o.leaves > 0) {
          std::vector<gra::M4Vec> lv;
          std::function<void(const gra::MDecayBranch &)> walk = [&](const gra::MDecayBranch &b) {
            if (b.legs.empty()) {
              lv.push_back(b.p4);
              return;
            }
            for (const auto &l : b.legs) walk(l);
          };
          for (const auto &b : proc->lts.decaytree) walk(b);
          for (int k = 0; k < o.leaves && k < static_cast<int>(lv.size()); ++k) {
            r[24 + 4 * k + 0] = lv[k].Px();
            r[24 + 4 * k + 1] = lv[k].Py();
            r[24 + 4 * k + 2] = lv[k].Pz();
            r[24 + 4 * k + 3] = lv[k].E();
          }
        }
      }
      write_doubles(ofile, out);
      return 0;
    }

    if (mode == "eikonal") {
      if (argc < 5) return 2;
      const std::string ofile = argv[4];
      const Opts        o     = parse_opts(argc, argv, 5);
      gra::MGraniitti   gen;
      setup(gen, card, process, o);
      gra::MProcess *proc = gen.proc;
      proc->post_Constructor();
      proc->Eikonal.S3Constructor(proc->GetMandelstam_s(), proc->GetInitialState(), false, o.nbt,
                                  o.nkt2);
      double tot = 0, el = 0, in = 0;
      proc->Eikonal.GetTotXS(tot, el, in);
      std::vector<double> out = {tot, el, in};
      const gra::IArray1D *arrs[2] = {&proc->Eikonal.MBT, &proc->Eikonal.MSA};
      for (const gra::IArray1D *a : arrs) {
        for (std::size_t i = 0; i < a->F.size_row(); ++i) {
          out.push_back(std::real(a->F[i][gra::IArray1D::X]));
          out.push_back(std::real(a->F[i][gra::IArray1D::Y]));
          out.push_back(std::imag(a->F[i][gra::IArray1D::Y]));
        }
      }
      write_doubles(ofile, out);
      std::printf("%.12e %.12e %.12e\n", tot, el, in);
      return 0;
    }

    if (mode == "vegas") {
      const Opts      o = parse_opts(argc, argv, 4);
      gra::MGraniitti gen;
      setup(gen, card, process, o);
      if (o.ncall > 0 || o.iter > 0 || o.precision > 0) {
        gra::VEGASPARAM vp;
        if (o.ncall > 0) vp.NCALL = o.ncall;
        if (o.iter > 0) vp.ITER = o.iter;
        if (o.precision > 0) vp.PRECISION = o.precision;
        gen.SetVegasParam(vp);
      }
      if (gen.proc->GetScreening()) {
        gen.proc->post_Constructor();
        gen.proc->Eikonal.S3Constructor(gen.proc->GetMandelstam_s(), gen.proc->GetInitialState(),
                                        false, o.nbt, o.nkt2);
      }
      gen.Initialize();
      double xs = 0, err = 0;
      gen.GetXS(xs, err);
      std::printf("RESULT %.12e %.12e\n", xs, err);
      return 0;
    }
  } catch (const std::exception &e) {
    std::fprintf(stderr, "reference threw: %s\n", e.what());
    return 4;
  }
  std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
