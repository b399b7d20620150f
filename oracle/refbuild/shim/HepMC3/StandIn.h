// Header-only stand-in for the small part of the HepMC3 3.2.0 interface that the
// event generator's library sources name. It exists only so that the reference
// sources compile into the test oracle; events are built in memory and the writers
// discard them. The event weight never depends on these types.
#ifndef GRN_HEPMC3_STANDIN_H
#define GRN_HEPMC3_STANDIN_H
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace HepMC3 {

class FourVector {
 public:
  FourVector() {}
  FourVector(double x, double y, double z, double e) : x_(x), y_(y), z_(z), e_(e) {}
  double x() const { return x_; }
  double y() const { return y_; }
  double z() const { return z_; }
  double e() const { return e_; }
  double px() const { return x_; }
  double py() const { return y_; }
  double pz() const { return z_; }
  double t() const { return e_; }

 private:
  double x_ = 0, y_ = 0, z_ = 0, e_ = 0;
};

struct Units {
  enum MomentumUnit { MEV, GEV };
  enum LengthUnit { MM, CM };
};

class Attribute {
 public:
  virtual ~Attribute() {}
};

class GenCrossSection : public Attribute {
 public:
  void set_cross_section(double xs, double err) {
    xs_  = xs;
    err_ = err;
  }

 private:
  double xs_ = 0, err_ = 0;
};

class GenParticle {
 public:
  GenParticle(const FourVector &p = FourVector(), int pdg = 0, int status = 0)
      : p_(p), pdg_(pdg), status_(status) {}
  const FourVector &momentum() const { return p_; }
  int               pid() const { return pdg_; }
  int               status() const { return status_; }

 private:
  FourVector p_;
  int        pdg_ = 0, status_ = 0;
};
typedef std::shared_ptr<GenParticle> GenParticlePtr;

class GenVertex {
 public:
  GenVertex(const FourVector &pos = FourVector()) : pos_(pos) {}
  void add_particle_in(const GenParticlePtr &p) { in_.push_back(p); }
  void add_particle_out(const GenParticlePtr &p) { out_.push_back(p); }

 private:
  FourVector                  pos_;
  std::vector<GenParticlePtr> in_, out_;
};
typedef std::shared_ptr<GenVertex> GenVertexPtr;

class GenRunInfo {
 public:
  struct ToolInfo {
    std::string name;
    std::string version;
    std::string description;
  };
  std::vector<ToolInfo> &tools() { return tools_; }

 private:
  std::vector<ToolInfo> tools_;
};

class GenEvent {
 public:
  GenEvent(Units::MomentumUnit = Units::GEV, Units::LengthUnit = Units::MM) {}
  void add_vertex(const GenVertexPtr &v) { vertices_.push_back(v); }
  void add_attribute(const std::string &name, const std::shared_ptr<Attribute> &a) {
    attributes_[name] = a;
  }
  std::vector<double> &weights() { return weights_; }

 private:
  std::vector<GenVertexPtr>                         vertices_;
  std::map<std::string, std::shared_ptr<Attribute>> attributes_;
  std::vector<double>                               weights_;
};

// Writers: accept events and drop them.
class WriterBase {
 public:
  explicit WriterBase(const std::string & = "", std::shared_ptr<GenRunInfo> = nullptr) {}
  virtual ~WriterBase() {}
  void write_event(const GenEvent &) {}
  void close() {}
  bool failed() { return false; }
};
class WriterAscii : public WriterBase {
 public:
  using WriterBase::WriterBase;
};
class WriterAsciiHepMC2 : public WriterBase {
 public:
  using WriterBase::WriterBase;
};
class WriterHEPEVT : public WriterBase {
 public:
  using WriterBase::WriterBase;
};

struct Print {
  static void listing(const GenEvent &) {}
  static void content(const GenEvent &) {}
};

}  // namespace HepMC3
#endif
