/* Plain-C description of one Monte Carlo system: box, pair model, atom-type
 * tables and Ewald settings. Shared by the GPU library (faunus_gb300.h) and
 * by the FP64 oracle used in tests, so both read the same numbers.
 *
 * Units follow the reference (Faunus): lengths in Angstrom, energies in kT.
 * Field-by-field provenance in the reference:
 *   bjerrum            Coulomb::lB, src/potentials.cpp:357-363 (pc::lB(epsr))
 *   type_charge        AtomData::charge, species.h:417
 *   type_sigma         AtomData::sigma (radius = sigma/2), species.h:413-415
 *   type_eps           AtomData::eps already in kT (species.h:293 converts kJ/mol)
 *   type_dp            AtomData::dp, the AtomicTranslation step, move.h:838-845
 *   ewald_*            NonbondedEwald JSON keys, ewald.h:507-530
 *   dh_debye_length    DebyeHuckel "debyelength", src/potentials.cpp:770-782
 */
#ifndef FG_PARAMS_H
#define FG_PARAMS_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Pair models (the reference's energy classes they stand in for). */
enum {
    /* NonbondedEwald<Tspace, WeeksChandlerAndersen> (ewald.h:228-757):
     * EwaldReal + WCA pairs, reciprocal Q(k), self and surface terms. */
    FG_MODEL_EWALD_WCA = 1,
    /* Nonbonded<Tspace, CombinedPairPotential<DebyeHuckel,
     * LennardJonesMixed<LorentzBerthelot>>> (energy.h:781-951). */
    FG_MODEL_DH_LJ = 2,
    /* NonbondedVector<Tspace, CoulombGalore + IonDipole + DipoleDipoleGalore
     * (reaction field) + LennardJonesMixed> for rigid dipolar molecules. */
    FG_MODEL_MULTIPOLE_RF = 3,
    /* NonbondedEwald<Tspace, LennardJonesLB, useIonIon, useIonDipole,
     * useDipoleDipole> on point charges and point dipoles (DipoleParticle):
     * EwaldReal + LJ pairs, reciprocal Q(k) of charges and dipoles, self and
     * surface terms (ewald.h:28-32, 203-216). */
    FG_MODEL_EWALD_DIPOLE = 4
};

/* ewald_terms bits: the useIonIon / useIonDipole / useDipoleDipole template
 * flags of NonbondedEwald (ewald.h:231). */
enum { FG_EWALD_ION_ION = 1, FG_EWALD_ION_DIPOLE = 2, FG_EWALD_DIPOLE_DIPOLE = 4 };

#define FG_MAX_TYPES 16

typedef struct fg_params {
    int32_t model;                    /* FG_MODEL_* */
    int32_t n_types;                  /* atom types used, <= FG_MAX_TYPES */
    double box[3];                    /* Cuboid side lengths (Angstrom) */
    double bjerrum;                   /* Bjerrum length lB (Angstrom) */
    double type_charge[FG_MAX_TYPES]; /* atom-type charge (e), used for the
                                         Ewald effective-charge ratio */
    double type_sigma[FG_MAX_TYPES];  /* LJ/WCA sigma (Angstrom) */
    double type_eps[FG_MAX_TYPES];    /* LJ/WCA epsilon (kT) */
    double type_dp[FG_MAX_TYPES];     /* translation parameter (Angstrom) */
    /* Ewald (FG_MODEL_EWALD_WCA) */
    double ewald_alpha;               /* damping alpha (1/Angstrom) */
    double ewald_cutoff;              /* real-space cutoff (Angstrom) */
    double ewald_cutoff_k;            /* "cutoffK": |n| <= cutoffK */
    double ewald_debye_length;        /* "debyelength" (kappa = 1/this) */
    double ewald_eps_surf;            /* surroundings; < 1 means tinfoil */
    int32_t ewald_spherical_sum;      /* 1 = spherical k-space sum */
    int32_t ewald_update_frequency;   /* full Q(k) rebuild after this many
                                         accepted moves (<=0: every accept) */
    /* Debye-Hueckel (FG_MODEL_DH_LJ) */
    double dh_debye_length;           /* 1/kappa (Angstrom) */
    /* Multipole reaction field (FG_MODEL_MULTIPOLE_RF) */
    double rf_cutoff;                 /* reaction-field cutoff (Angstrom) */
    double rf_eps_rf;                 /* dielectric of the continuum beyond rc */
    double rf_eps_r;                  /* dielectric inside the cavity */
    /* Temperature scale: Boltzmann factors use dU / kT_scale (1 = the
     * reference's convention of energies already in kT). */
    double kT_scale;
    /* GPU execution options (the oracle ignores them) */
    int32_t use_cell_list;            /* 1 = cell list for the real-space sum */
    /* Dipolar Ewald (FG_MODEL_EWALD_DIPOLE) */
    int32_t ewald_terms;              /* FG_EWALD_* bits */
    int32_t ewald_dipole_quirk;       /* 0: the Ewald sum as ewald.h:28-32 and
                                         203-216 state it (real-space ion-dipole
                                         and dipole-dipole terms, reciprocal
                                         |Q_ion + Q_dip|^2); 1: as the reference's
                                         live code computes it: EwaldReal returns
                                         after its ion-ion term (ewald.h:109-110)
                                         and the reciprocal cross term is
                                         2 Re(Q_ion Q_dip) (ewald.h:304-305) */
    int32_t ewald_isotropic_pbc;      /* "isotropic_pbc" (ewald.h:525): k-vectors
                                         with n_x, n_y, n_z >= 0, a factor 2 per
                                         positive component, and the real
                                         Q(k) = sum q eff cos(k_x x) cos(k_y y)
                                         cos(k_z z) (ewald.h:347-360, 394-399);
                                         FG_MODEL_EWALD_WCA only */
    int32_t reserved[4];
} fg_params;

#ifdef __cplusplus
}
#endif
#endif
