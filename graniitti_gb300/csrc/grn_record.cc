// grn_record.cc — event records of accepted points in the generator's output formats.
//
// The layout follows MProcess::CommonRecord (src/MProcess.cc:1588-1680): four vertices
//   v1: beam1 -> forward proton 1 + propagator q1
//   v2: beam2 -> forward proton 2 + propagator q2
//   v3: q1 + q2 -> central system (PDG 90)
//   v4: central system -> the two central final states
// with status codes beam 4, stable 1, intermediate 81 (include/Graniitti/MPDG.h:42-50),
// the cross section in pb and the event weight with every event, as MGraniitti::SaveEvent
// writes them (src/MGraniitti.cc:1665-1715). The three text layouts are those of HepMC3's
// ASCII v3 writer, HepMC2's IO_GenEvent and HEPEVT, produced here directly.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "graniitti_gb300.h"

namespace {

struct Particle {
  int    pdg, status;
  double p[4];  // px, py, pz, E
  double m;
};

// Invariant mass with the sign convention of a space-like propagator kept (m = -sqrt(-m2)).
double mass_of(const double *p) {
  const double m2 = p[3] * p[3] - p[0] * p[0] - p[1] * p[1] - p[2] * p[2];
  return m2 >= 0 ? std::sqrt(m2) : -std::sqrt(-m2);
}

}  // namespace

struct grn_writer {
  FILE       *fp     = nullptr;
  int         format = GRN_FORMAT_HEPMC3;
  int64_t     events = 0;
};

extern "C" {

grn_status grn_writer_open(const char *path, int32_t format, const char *tool, const char *card,
                           grn_writer **out) {
  if (!path || !out) return GRN_ERR_INVALID;
  *out = nullptr;
  if (format != GRN_FORMAT_HEPMC3 && format != GRN_FORMAT_HEPMC2 && format != GRN_FORMAT_HEPEVT)
    return GRN_ERR_INVALID;
  FILE *fp = std::fopen(path, "w");
  if (!fp) return GRN_ERR_INVALID;
  auto *w   = new grn_writer();
  w->fp     = fp;
  w->format = format;
  if (format == GRN_FORMAT_HEPMC3) {
    std::fprintf(fp, "HepMC::Version 3.02.06\nHepMC::Asciiv3-START_EVENT_LISTING\n");
    std::fprintf(fp, "W Default\n");
    std::fprintf(fp, "T %s\\|%s\\|Generator\n", tool ? tool : "GRANIITTI", grn_version());
    if (card) std::fprintf(fp, "T %s\\|1.0\\|Steering card\n", card);
  } else if (format == GRN_FORMAT_HEPMC2) {
    std::fprintf(fp, "\nHepMC::Version 2.06.09\nHepMC::IO_GenEvent-START_EVENT_LISTING\n");
  }
  *out = w;
  return GRN_OK;
}

grn_status grn_writer_close(grn_writer *w) {
  if (!w) return GRN_OK;
  if (w->fp) {
    if (w->format == GRN_FORMAT_HEPMC3)
      std::fprintf(w->fp, "HepMC::Asciiv3-END_EVENT_LISTING\n\n");
    else if (w->format == GRN_FORMAT_HEPMC2)
      std::fprintf(w->fp, "HepMC::IO_GenEvent-END_EVENT_LISTING\n");
    std::fclose(w->fp);
  }
  delete w;
  return GRN_OK;
}

grn_status grn_write_records(grn_writer *w, const double *p4, int64_t n, const int32_t pdg[3],
                             const double mass[3], double sqrt_s, double weight, double sigma_pb,
                             double sigma_err_pb) {
  if (!w || !w->fp || !pdg || !mass || n < 0 || (n > 0 && !p4) || !(sqrt_s > 2 * mass[0]))
    return GRN_ERR_INVALID;
  // beams along +-z with equal energies (symmetric beams only, as the engine)
  const double Eb = 0.5 * sqrt_s, mb = mass[0];
  const double pz = std::sqrt(std::max(Eb * Eb - mb * mb, 0.0));
  FILE        *fp = w->fp;
  for (int64_t i = 0; i < n; ++i) {
    const double *q = &p4[static_cast<size_t>(i) * 16];
    Particle      part[9];
    part[0] = {pdg[0], 4, {0.0, 0.0, pz, Eb}, mb};           // beam 1
    part[1] = {pdg[0], 1, {q[0], q[1], q[2], q[3]}, mb};      // forward 1
    part[3] = {pdg[0], 4, {0.0, 0.0, -pz, Eb}, mb};          // beam 2
    part[4] = {pdg[0], 1, {q[4], q[5], q[6], q[7]}, mb};      // forward 2
    part[7] = {pdg[1], 1, {q[8], q[9], q[10], q[11]}, mass[1]};
    part[8] = {pdg[2], 1, {q[12], q[13], q[14], q[15]}, mass[2]};
    Particle q1{99, 81, {}, 0.0}, q2{99, 81, {}, 0.0}, X{90, 81, {}, 0.0};
    for (int k = 0; k < 4; ++k) {
      q1.p[k] = part[0].p[k] - part[1].p[k];
      q2.p[k] = part[3].p[k] - part[4].p[k];
      X.p[k]  = part[7].p[k] + part[8].p[k];
    }
    q1.m = mass_of(q1.p);
    q2.m = mass_of(q2.p);
    X.m  = mass_of(X.p);
    part[2] = q1;
    part[5] = q2;
    part[6] = X;
    const int64_t ev = w->events++;
    if (w->format == GRN_FORMAT_HEPMC3) {
      // particles numbered in the order CommonRecord adds its vertices; a particle made at
      // a vertex with one incoming particle names that particle as its parent
      static const int parent[9] = {0, 1, 1, 0, 4, 4, -3, 7, 7};
      std::fprintf(fp, "E %lld 4 9\nU GEV MM\nW %.16e\n", static_cast<long long>(ev), weight);
      std::fprintf(fp, "A 0 GenCrossSection %.16e %.16e -1 -1\n", sigma_pb, sigma_err_pb);
      for (int k = 0; k < 9; ++k) {
        if (k == 6) std::fprintf(fp, "V -3 0 [3,6]\n");
        const Particle &a = part[k];
        std::fprintf(fp, "P %d %d %d %.16e %.16e %.16e %.16e %.16e %d\n", k + 1, parent[k], a.pdg,
                     a.p[0], a.p[1], a.p[2], a.p[3], a.m, a.status);
      }
    } else if (w->format == GRN_FORMAT_HEPMC2) {
      // vertices -1..-4; beams are the orphan incoming particles of v1, v2
      static const int end_vtx[9] = {-1, 0, -3, -2, 0, -3, -4, 0, 0};
      std::fprintf(fp, "E %lld -1 -1.0000000000000000e+00 -1.0000000000000000e+00 "
                       "-1.0000000000000000e+00 0 -3 4 1 4 0 1 %.16e\n",
                   static_cast<long long>(ev), weight);
      std::fprintf(fp, "N 1 \"Default\"\nU GEV MM\nC %.16e %.16e\n", sigma_pb, sigma_err_pb);
      auto pline = [&](int k) {
        const Particle &a = part[k];
        std::fprintf(fp, "P %d %d %.16e %.16e %.16e %.16e %.16e %d 0 0 %d 0\n", k + 1, a.pdg,
                     a.p[0], a.p[1], a.p[2], a.p[3], a.m, a.status, end_vtx[k]);
      };
      std::fprintf(fp, "V -1 0 0 0 0 0 1 2 0\n");
      pline(0), pline(1), pline(2);
      std::fprintf(fp, "V -2 0 0 0 0 0 1 2 0\n");
      pline(3), pline(4), pline(5);
      std::fprintf(fp, "V -3 0 0 0 0 0 0 1 0\n");
      pline(6);
      std::fprintf(fp, "V -4 0 0 0 0 0 0 2 0\n");
      pline(7), pline(8);
    } else {
      // HEPEVT: status, id, first/last mother, first/last daughter (1-based), p, m
      static const int mo[9][2] = {{0, 0}, {1, 1}, {1, 1}, {0, 0}, {4, 4},
                                   {4, 4}, {3, 6}, {7, 7}, {7, 7}};
      static const int da[9][2] = {{2, 3}, {0, 0}, {7, 7}, {5, 6}, {0, 0},
                                   {7, 7}, {8, 9}, {0, 0}, {0, 0}};
      std::fprintf(fp, "E % 12lld% 12d\n", static_cast<long long>(ev), 9);
      for (int k = 0; k < 9; ++k) {
        const Particle &a = part[k];
        std::fprintf(fp, "% 12d% 12d% 12d% 12d% 12d% 12d% 19.8E% 19.8E% 19.8E% 19.8E% 19.8E\n",
                     a.status, a.pdg, mo[k][0], mo[k][1], da[k][0], da[k][1], a.p[0], a.p[1],
                     a.p[2], a.p[3], a.m);
      }
    }
  }
  std::fflush(fp);
  return GRN_OK;
}

grn_status grn_write_events(grn_writer *w, grn_engine *e, const double *u, int64_t n,
                            const int32_t pdg[3], double weight, double sigma_pb,
                            double sigma_err_pb, int64_t *written) {
  if (written) *written = 0;
  if (!w || !w->fp || !e || !pdg || n < 0 || (n > 0 && !u)) return GRN_ERR_INVALID;
  if (n == 0) return GRN_OK;
  const grn_process_params *P = grn_engine_params(e);
  std::vector<double>       p4(static_cast<size_t>(n) * 16), ts(static_cast<size_t>(n) * 2);
  std::vector<uint8_t>      fl(static_cast<size_t>(n));
  const grn_status st = grn_event_kinematics(e, u, n, grn_dim(e), p4.data(), ts.data(), fl.data());
  if (st != GRN_OK) return st;
  // keep the points whose kinematics passed
  int64_t m = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (!(fl[i] & GRN_FLAG_KINEMATICS_OK)) continue;
    if (m != i) std::copy(&p4[i * 16], &p4[i * 16] + 16, &p4[m * 16]);
    ++m;
  }
  const double mass[3] = {P->m_beam, P->m_central[0], P->m_central[1]};
  const grn_status st2 = grn_write_records(w, p4.data(), m, pdg, mass, P->sqrt_s, weight, sigma_pb,
                                           sigma_err_pb);
  if (st2 == GRN_OK && written) *written = m;
  return st2;
}

}  // extern "C"
