// Test stand-in for NBodylib's NBody.h: just enough of NBody::Particle, NBody::System,
// NBody::Coordinate and NBody::Matrix (the accessors include/nbkdt/KDTree.h uses) to compile and run the
// drop-in KDTree where NBodylib itself is not installed. The member layout follows the
// reference's default Particle (88 bytes: mass, position[3], velocity[3], pid, id, type,
// rho, phi).
#pragma once
#include <cmath>
#include <cstddef>
#include <vector>

typedef double Double_t;
typedef int Int_t;

namespace NBody {

class Coordinate {
 public:
  Coordinate(Double_t x = 0, Double_t y = 0, Double_t z = 0) {
    c_[0] = x;
    c_[1] = y;
    c_[2] = z;
  }
  Double_t* GetCoord() { return c_; }
  Double_t operator[](int i) const { return c_[i]; }

 private:
  Double_t c_[3];
};

class Matrix {
 public:
  Matrix() {
    for (int i = 0; i < 9; i++) m_[i] = 0;
  }
  explicit Matrix(const Double_t m[9]) {
    for (int i = 0; i < 9; i++) m_[i] = m[i];
  }
  Double_t& operator()(int i, int j) { return m_[j + 3 * i]; }
  const Double_t& operator()(int i, int j) const { return m_[j + 3 * i]; }

 private:
  Double_t m_[9];
};

class Particle {
 public:
  Particle() = default;
  Double_t GetMass() const { return mass_; }
  void SetMass(Double_t m) { mass_ = m; }
  Double_t GetPosition(int j) const { return pos_[j]; }
  const Double_t* GetPosition() const { return pos_; }
  void SetPosition(int j, Double_t v) { pos_[j] = v; }
  Double_t GetVelocity(int j) const { return vel_[j]; }
  void SetVelocity(int j, Double_t v) { vel_[j] = v; }
  Int_t GetID() const { return id_; }
  void SetID(const Int_t& i) { id_ = i; }
  Int_t GetPID() const { return pid_; }
  void SetPID(const Int_t& i) { pid_ = i; }
  Double_t GetDensity() const { return rho_; }
  void SetDensity(const Double_t& r) { rho_ = r; }

 private:
  Double_t mass_ = 0;
  Double_t pos_[3] = {0, 0, 0};
  Double_t vel_[3] = {0, 0, 0};
  Int_t pid_ = 0, id_ = 0, type_ = 0;
  Double_t rho_ = 0, phi_ = 0;
};

class System {
 public:
  // as the reference's System(num, p, t, period) (src/NBody/System.h:60): the system keeps
  // its own copy of the particles
  System(Int_t num, Particle* p, Double_t t = 0.0, Double_t* period = NULL)
      : parts_(p, p + num), period_(period ? period[0] : 0, period ? period[1] : 0,
                                    period ? period[2] : 0) {
    (void)t;
  }
  Particle* Parts() { return parts_.data(); }
  Int_t GetNumParts() const { return (Int_t)parts_.size(); }
  Coordinate GetPeriod() const { return period_; }
  Particle& operator[](Int_t i) { return parts_[i]; }

 private:
  std::vector<Particle> parts_;
  Coordinate period_;
};

}  // namespace NBody
