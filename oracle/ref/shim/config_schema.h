// Hand-written stand-in for the Regent-generated config header, limited to
// the fields that the mixture constructors (`Mix(const Config&)`) read.
// Test infrastructure only: it lets the reference's CPU task code build
// without the Regent toolchain.
#ifndef HTR_ORACLE_CONFIG_SCHEMA_STUB_H
#define HTR_ORACLE_CONFIG_SCHEMA_STUB_H

#include <stdint.h>

enum { MixtureModel_ConstPropMix = 0, MixtureModel_AirMix = 1, MixtureModel_IsentropicMix = 2 };
enum { ViscosityModel_Constant = 0, ViscosityModel_PowerLaw = 1, ViscosityModel_Sutherland = 2 };

struct Species {
  char Name[10];
  double MolarFrac;
};

struct Mixture {
  struct {
    uint32_t length;
    struct Species values[20];
  } Species;
};

struct HTRStubViscosityModel {
  int type;
  struct {
    struct { double Visc; } Constant;
    struct { double TempRef; double ViscRef; } PowerLaw;
    struct { double SRef; double TempRef; double ViscRef; } Sutherland;
  } u;
};

struct Config {
  struct {
    struct {
      int type;
      struct {
        struct {
          double gasConstant;
          double gamma;
          double prandtl;
          struct HTRStubViscosityModel viscosityModel;
        } ConstPropMix;
        struct {
          double PRef;
          double TRef;
          double LRef;
          struct Mixture XiRef;
        } AirMix;
      } u;
    } mixture;
  } Flow;
};

#endif
