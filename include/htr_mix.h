/* Mixture descriptors accepted by the htr_gb300 C ABI.
 *
 * Each struct is byte-compatible with the `struct Mix` that HTR compiles for
 * the corresponding equation of state, so a caller that already holds the
 * reference's task argument (`Args::mix`) can pass its address unchanged:
 *
 *   htr_constpropmix_t  <->  src/Mixtures/ConstPropMix.hpp:98-112   (EOS=ConstPropMix)
 *   htr_airmix_t        <->  src/Mixtures/MultiComponent.hpp:109-140 with the
 *                            AirMix sizes of src/Mixtures/AirMix.hpp:35-53
 *                            (5 species, 2 standard + 3 third-body reactions,
 *                            3 NASA-9 ranges, no ions, mass-action orders)
 *
 * Member types, order and padding follow the reference (float switch
 * temperatures, float stoichiometric coefficients and Arrhenius exponents),
 * because the arithmetic promotes those floats exactly where the reference
 * does.  The layout is checked against the reference headers by the test
 * suite.
 */
#ifndef HTR_MIX_H
#define HTR_MIX_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Equation-of-state selector (the reference selects it at compile time with
 * -DEOS=..., src/prometeo_const.h:39-43). */
enum htr_eos {
  HTR_EOS_CONSTPROPMIX = 1, /* single-species calorically perfect gas */
  HTR_EOS_AIRMIX = 2        /* 5-species air, Park-type kinetics */
};

/* ConstPropMix viscosity laws (config_schema.lua ViscosityModel union). */
enum htr_viscosity_model {
  HTR_VISC_CONSTANT = 0,
  HTR_VISC_POWERLAW = 1,
  HTR_VISC_SUTHERLAND = 2
};

typedef struct {
  double R;
  double gamma;
  int viscosityModel;
  double constantVisc;
  double powerlawTempRef;
  double powerlawViscRef;
  double sutherlandSRef;
  double sutherlandTempRef;
  double sutherlandViscRef;
  double Prandtl;
} htr_constpropmix_t;

#define HTR_AIR_NSPEC 5
#define HTR_AIR_NREAC 2
#define HTR_AIR_NTBREAC 3
#define HTR_AIR_MAX_REACTANTS 2
#define HTR_AIR_MAX_PRODUCTS 2
#define HTR_AIR_MAX_TB 5

/* NASA 9-coefficient polynomials in three temperature ranges
 * (src/Mixtures/Species.hpp:80-89). */
typedef struct {
  float TSwitch1;
  float TSwitch2;
  float TMin;
  float TMax;
  double cpH[9];
  double cpM[9];
  double cpL[9];
} htr_nasa9_t;

/* Lennard-Jones / Stockmayer transport data (Species.hpp:91-98). */
typedef struct {
  uint8_t Geom; /* 0 atom, 1 linear, 3 non-linear */
  double sigma;
  double kbOveps;
  double mu;
  double alpha;
  double Z298;
} htr_ljdata_t;

typedef struct {
  char Name[10];
  double W;
  uint8_t inx;
  htr_nasa9_t cpCoeff;
  htr_ljdata_t DiffCoeff;
} htr_species_t;

typedef struct {
  double A;
  float n;
  float EovR;
} htr_arrhenius_t;

typedef struct {
  uint8_t ind;
  float nu;
} htr_stoich_t;

typedef struct {
  uint8_t ind;
  float eff;
} htr_collider_t;

typedef struct {
  htr_arrhenius_t ArrCoeff;
  bool has_backward;
  uint8_t Neducts;
  uint8_t Npducts;
  htr_stoich_t educts[HTR_AIR_MAX_REACTANTS];
  htr_stoich_t pducts[HTR_AIR_MAX_PRODUCTS];
} htr_reaction_t;

typedef struct {
  htr_arrhenius_t ArrCoeff;
  bool has_backward;
  uint8_t Neducts;
  uint8_t Npducts;
  uint8_t Nthirdb;
  htr_stoich_t educts[HTR_AIR_MAX_REACTANTS];
  htr_stoich_t pducts[HTR_AIR_MAX_PRODUCTS];
  htr_collider_t thirdb[HTR_AIR_MAX_TB];
} htr_tbreaction_t;

typedef struct {
  htr_species_t species[HTR_AIR_NSPEC];
  htr_reaction_t reactions[HTR_AIR_NREAC];
  htr_tbreaction_t ThirdbodyReactions[HTR_AIR_NTBREAC];
  double PRef;
  double TRef;
  double XiRef[HTR_AIR_NSPEC];
  double MixWRef;
  double iMixWRef;
  double rhoRef;
  double ieRef;
  double iuRef;
  double iCpRef;
  double imuRef;
  double ilamRef;
  double iDiRef;
  double iwiRef;
  double iKiRef;
  double Eps0;
  double TMax;
  double TMin;
} htr_airmix_t;

#ifdef __cplusplus
}
#endif

#endif /* HTR_MIX_H */
