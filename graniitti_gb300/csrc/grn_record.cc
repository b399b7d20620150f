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

namespace {

// One event as a tree: particles (1-based in the text formats) with their production and
// end vertices; vertex v has incoming particles vin[v].
struct Tree {
  Particle part[13];
  int      np = 0, nv = 0;
  int      prod[13] = {}, end[13] = {};  // vertex numbers 1.., 0: none
  int      vin[7][2] = {}, nin[7] = {};
  int      add(const Particle &q, int prod_vtx) {
    part[np]  = q;
    prod[np]  = prod_vtx;
    return np++;
  }
  void link(int v, int in) {  // particle `in` (0-based) enters vertex v
    vin[v][nin[v]++] = in;
    end[in]          = v;
  }
};

// CommonRecord layout: beams -> forward legs + propagators, propagators -> system (90),
// system -> central pair, and for cascades each central particle (status 2, PDG_DECAY) -> its
// two daughters (WriteDecayKinematics, src/MProcess.cc:1289-1315).
Tree build_tree(const double *q, const double *d, const int32_t *pdg, const double *mass,
                double sqrt_s) {
  const double Eb = 0.5 * sqrt_s, mb = mass[0];
  const double pz = std::sqrt(std::max(Eb * Eb - mb * mb, 0.0));
  Tree t;
  const int b1 = t.add({pdg[0], 4, {0.0, 0.0, pz, Eb}, mb}, 0);
  t.nv = 1;
  t.link(1, b1);
  t.add({pdg[0], 1, {q[0], q[1], q[2], q[3]}, mb}, 1);
  const int q1 = t.add({99, 81, {}, 0.0}, 1);
  const int b2 = t.add({pdg[0], 4, {0.0, 0.0, -pz, Eb}, mb}, 0);
  t.nv = 2;
  t.link(2, b2);
  t.add({pdg[0], 1, {q[4], q[5], q[6], q[7]}, mb}, 2);
  const int q2 = t.add({99, 81, {}, 0.0}, 2);
  t.nv = 3;
  t.link(3, q1);
  t.link(3, q2);
  const int X = t.add({90, 81, {}, 0.0}, 3);
  t.nv = 4;
  t.link(4, X);
  const int st = d ? 2 : 1;
  const int c1 = t.add({pdg[1], st, {q[8], q[9], q[10], q[11]}, mass[1]}, 4);
  const int c2 = t.add({pdg[2], st, {q[12], q[13], q[14], q[15]}, mass[2]}, 4);
  for (int k = 0; k < 4; ++k) {
    t.part[q1].p[k] = t.part[b1].p[k] - t.part[1].p[k];
    t.part[q2].p[k] = t.part[b2].p[k] - t.part[4].p[k];
    t.part[X].p[k]  = t.part[c1].p[k] + t.part[c2].p[k];
  }
  t.part[q1].m = mass_of(t.part[q1].p);
  t.part[q2].m = mass_of(t.part[q2].p);
  t.part[X].m  = mass_of(t.part[X].p);
  if (d) {
    t.part[c1].m = mass_of(t.part[c1].p);  // off-shell masses
    t.part[c2].m = mass_of(t.part[c2].p);
    for (int c = 0; c < 2; ++c) {
      t.nv += 1;
      t.link(t.nv, c ? c2 : c1);
      for (int k = 0; k < 2; ++k) {
        const double *v = d + 4 * (2 * c + k);
        t.add({pdg[3 + 2 * c + k], 1, {v[0], v[1], v[2], v[3]}, mass[3 + 2 * c + k]}, t.nv);
      }
    }
  }
  return t;
}

// N-body central states: system (90) -> the nc central particles (status 1). q holds the
// forward legs (8 doubles), c the central particles (4 nc).
Tree build_tree_n(const double *q, const double *c, int nc, const int32_t *pdg,
                  const double *mass, double sqrt_s) {
  double q2[16];
  for (int k = 0; k < 8; ++k) q2[k] = q[k];
  for (int k = 0; k < 8; ++k) q2[8 + k] = c[k];
  const int32_t pdg2[3]  = {pdg[0], pdg[1], pdg[2]};
  const double  mass2[3] = {mass[0], mass[1], mass[2]};
  Tree t = build_tree(q2, nullptr, pdg2, mass2, sqrt_s);
  // the system is the sum of all of them; the others join the same vertex
  const int X = 6;
  for (int k = 0; k < 4; ++k) {
    double v = 0.0;
    for (int j = 0; j < nc; ++j) v += c[4 * j + k];
    t.part[X].p[k] = v;
  }
  t.part[X].m = mass_of(t.part[X].p);
  for (int j = 2; j < nc; ++j)
    t.add({pdg[1 + j], 1, {c[4 * j], c[4 * j + 1], c[4 * j + 2], c[4 * j + 3]}, mass[1 + j]}, 4);
  return t;
}

void write_tree(grn_writer *w, const Tree &t, double weight, double sigma_pb, double err_pb) {
  FILE         *fp = w->fp;
  const int64_t ev = w->events++;
  if (w->format == GRN_FORMAT_HEPMC3) {
    std::fprintf(fp, "E %lld %d %d\nU GEV MM\nW %.16e\n", static_cast<long long>(ev), t.nv, t.np,
                 weight);
    std::fprintf(fp, "A 0 GenCrossSection %.16e %.16e -1 -1\n", sigma_pb, err_pb);
    for (int k = 0; k < t.np; ++k) {
      // a particle made at a vertex with one incoming particle names that particle as its
      // parent; a vertex with several is written explicitly before its first product
      const int v = t.prod[k];
      int parent  = 0;
      if (v > 0 && t.nin[v] == 1) {
        parent = t.vin[v][0] + 1;
      } else if (v > 0) {
        bool first = true;
        for (int j = 0; j < k; ++j) first &= t.prod[j] != v;
        if (first) std::fprintf(fp, "V -%d 0 [%d,%d]\n", v, t.vin[v][0] + 1, t.vin[v][1] + 1);
        parent = -v;
      }
      const Particle &a = t.part[k];
      std::fprintf(fp, "P %d %d %d %.16e %.16e %.16e %.16e %.16e %d\n", k + 1, parent, a.pdg,
                   a.p[0], a.p[1], a.p[2], a.p[3], a.m, a.status);
    }
  } else if (w->format == GRN_FORMAT_HEPMC2) {
    // vertices -1.. -nv; the beams are the orphan incoming particles of v1, v2
    std::fprintf(fp, "E %lld -1 -1.0000000000000000e+00 -1.0000000000000000e+00 "
                     "-1.0000000000000000e+00 0 -3 %d 1 4 0 1 %.16e\n",
                 static_cast<long long>(ev), t.nv, weight);
    std::fprintf(fp, "N 1 \"Default\"\nU GEV MM\nC %.16e %.16e\n", sigma_pb, err_pb);
    auto pline = [&](int k) {
      const Particle &a = t.part[k];
      std::fprintf(fp, "P %d %d %.16e %.16e %.16e %.16e %.16e %d 0 0 %d 0\n", k + 1, a.pdg,
                   a.p[0], a.p[1], a.p[2], a.p[3], a.m, a.status, t.end[k] ? -t.end[k] : 0);
    };
    for (int v = 1; v <= t.nv; ++v) {
      int n_orphan = 0, n_out = 0;
      for (int k = 0; k < t.np; ++k) {
        n_orphan += (t.prod[k] == 0 && t.end[k] == v);
        n_out += (t.prod[k] == v);
      }
      std::fprintf(fp, "V -%d 0 0 0 0 0 %d %d 0\n", v, n_orphan, n_out);
      for (int k = 0; k < t.np; ++k)
        if (t.prod[k] == 0 && t.end[k] == v) pline(k);
      for (int k = 0; k < t.np; ++k)
        if (t.prod[k] == v) pline(k);
    }
  } else {
    // HEPEVT: status, id, first/last mother, first/last daughter (1-based), p, m
    std::fprintf(fp, "E % 12lld% 12d\n", static_cast<long long>(ev), t.np);
    for (int k = 0; k < t.np; ++k) {
      const Particle &a = t.part[k];
      int mo[2] = {0, 0}, da[2] = {0, 0};
      const int v = t.prod[k];
      if (v > 0) {
        mo[0] = t.vin[v][0] + 1;
        mo[1] = t.vin[v][t.nin[v] - 1] + 1;
      }
      if (t.end[k] > 0) {
        for (int j = 0; j < t.np; ++j)
          if (t.prod[j] == t.end[k]) {
            if (!da[0]) da[0] = j + 1;
            da[1] = j + 1;
          }
      }
      std::fprintf(fp, "% 12d% 12d% 12d% 12d% 12d% 12d% 19.8E% 19.8E% 19.8E% 19.8E% 19.8E\n",
                   a.status, a.pdg, mo[0], mo[1], da[0], da[1], a.p[0], a.p[1], a.p[2], a.p[3],
                   a.m);
    }
  }
}

}  // namespace

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
  for (int64_t i = 0; i < n; ++i)
    write_tree(w, build_tree(&p4[static_cast<size_t>(i) * 16], nullptr, pdg, mass, sqrt_s),
               weight, sigma_pb, sigma_err_pb);
  std::fflush(w->fp);
  return GRN_OK;
}

grn_status grn_write_cascade_records(grn_writer *w, const double *p4, const double *pd, int64_t n,
                                     const int32_t pdg[7], const double mass[7], double sqrt_s,
                                     double weight, double sigma_pb, double sigma_err_pb) {
  if (!w || !w->fp || !pdg || !mass || n < 0 || (n > 0 && (!p4 || !pd)) ||
      !(sqrt_s > 2 * mass[0]))
    return GRN_ERR_INVALID;
  for (int64_t i = 0; i < n; ++i)
    write_tree(w,
               build_tree(&p4[static_cast<size_t>(i) * 16], &pd[static_cast<size_t>(i) * 16],
                          pdg, mass, sqrt_s),
               weight, sigma_pb, sigma_err_pb);
  std::fflush(w->fp);
  return GRN_OK;
}

grn_status grn_write_events(grn_writer *w, grn_engine *e, const double *u, int64_t n,
                            const int32_t *pdg, int32_t n_pdg, double weight, double sigma_pb,
                            double sigma_err_pb, int64_t *written) {
  if (written) *written = 0;
  if (!w || !w->fp || !e || !pdg || n < 0 || (n > 0 && !u)) return GRN_ERR_INVALID;
  const grn_process_params *P = grn_engine_params(e);
  const int  nc   = P->n_central;
  const bool casc = P->n_decay == 2, four = nc >= 4;  // four: an N-body central state
  if (n_pdg != (casc ? 7 : (four ? 1 + nc : 3))) return GRN_ERR_INVALID;
  if (n == 0) return GRN_OK;
  const int dim = grn_dim(e);
  std::vector<double>  p4(static_cast<size_t>(n) * 16), ts(static_cast<size_t>(n) * 2);
  const size_t per = four ? static_cast<size_t>(4 * nc) : 16;  // daughters' doubles per point
  std::vector<double>  pd((casc || four) ? static_cast<size_t>(n) * per : 0);
  std::vector<uint8_t> fl(static_cast<size_t>(n));
  grn_status st = grn_event_kinematics(e, u, n, dim, p4.data(), ts.data(), fl.data());
  if (st == GRN_OK && (casc || four)) st = grn_event_daughters(e, u, n, dim, pd.data());
  if (st != GRN_OK) return st;
  // keep the points whose kinematics passed
  int64_t m = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (!(fl[i] & GRN_FLAG_KINEMATICS_OK)) continue;
    if (m != i) {
      std::copy(&p4[i * 16], &p4[i * 16] + 16, &p4[m * 16]);
      if (casc || four) std::copy(&pd[i * per], &pd[i * per] + per, &pd[m * per]);
    }
    ++m;
  }
  if (four) {
    double mass[7] = {P->m_beam};
    for (int k = 0; k < nc; ++k) mass[1 + k] = P->m_central[k];
    if (!(P->sqrt_s > 2 * mass[0])) return GRN_ERR_INVALID;
    for (int64_t i = 0; i < m; ++i)
      write_tree(w, build_tree_n(&p4[i * 16], &pd[i * per], nc, pdg, mass, P->sqrt_s), weight,
                 sigma_pb, sigma_err_pb);
    std::fflush(w->fp);
  } else if (casc) {
    const double mass[7] = {P->m_beam,       P->m_central[0],  P->m_central[1], P->m_daughter[0],
                            P->m_daughter[1], P->m_daughter[2], P->m_daughter[3]};
    st = grn_write_cascade_records(w, p4.data(), pd.data(), m, pdg, mass, P->sqrt_s, weight,
                                   sigma_pb, sigma_err_pb);
  } else {
    const double mass[3] = {P->m_beam, P->m_central[0], P->m_central[1]};
    st = grn_write_records(w, p4.data(), m, pdg, mass, P->sqrt_s, weight, sigma_pb,
                           sigma_err_pb);
  }
  if (st == GRN_OK && written) *written = m;
  return st;
}

}  // extern "C"
