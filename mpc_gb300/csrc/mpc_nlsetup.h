// mpc_nlsetup.h -- host-side setup of the fused nonlinear step's constants, shared by the
// context-based entry points (mpc_capi.cu) and the allocation-free one (mpc_noalloc.cu).
//
// Gas tables (plasma.c:4-40 ionizpot, plasma.c:61-115 Natoms), the ADK prefactors with
// n*_q = q / sqrt(2 Ip_q) and C_nl from 2^(2 n*) (plasma.c:162-175, corrected), the Drude terms
// with the drift velocity from w0 alone (plasma.c:196-213, corrected), all in FP64, rounded once
// to the FP32 constants of NLConst (mpc_kernels.cuh).
#pragma once
#include <math.h>
#include <string.h>

#include "../../include/mpc_gpu.h"
#include "mpc_kernels.cuh"

namespace mpc {

// constants.h:1-11
constexpr double kZW0 = 377.0, kNC = 1.0, kFCTR = 0.89, kIH = 27.21, kEF = 5.14220642e11;
constexpr double kME = 9.1094e-31, kEL0 = 1.602e-19, kNAVO = 6.02214e+23, kT0 = 2.4188843265e-17;
constexpr double kC0 = 299792458.0, kHBAR = 1.054560652926899e-34;
// device units: |a|^2 = intensity / kIUnit
constexpr double kIUnit = 1e16;

// ionizpot (plasma.c:4-40) and Natoms (plasma.c:61-115); the xenon molar mass 5.761 is kept as
// the reference writes it.  Returns 0 for an unknown gas.  `gas` is read up to 9 characters
// (the reference's char gas[9]).
inline int gas_tables(const char* gas, double* I1, double* I2, double* Natm, double* sig) {
    struct G { const char* n; double i1, i2, dens, M, sig; };
    static const G g[] = {
        {"Argon", 15.75962, 27.62967, 1.784 * 1e3, 39.941, 1.57e-20},
        {"Helium", 24.58741, 54.41778, 0.166e3, 4.002602, 6.11e-20},
        {"Neon", 21.5646, 40.96328, 0.9002e3, 20.1797, 1.65e-20},
        {"Air", 0.78084 * 14.53414 + 0.20946 * 13.61806 + 0.00934 * 15.75962,
         0.78084 * 29.6013 + 0.20946 * 35.11730 + 0.00934 * 27.62967, 1.205e3, 28.97, 10e-20},
        {"Nitrogen", 14.53414, 29.6013, 1.65e3, 14.0067, 10.2e-20},
        {"Xenon", 12.1298, 21.20979, 5.86e3, 5.761, 3.55e-20},
        {"Krypton", 13.99961, 24.35985, 3.749e3, 83.798, 1.15e-20},
    };
    for (const G& e : g)
        if (strncmp(gas, e.n, 9) == 0) {
            *I1 = e.i1;
            *I2 = e.i2;
            *Natm = e.dens * kNAVO / e.M;
            *sig = e.sig;
            return 1;
        }
    return 0;
}

// The nonlinear step's constants for the device units a = A * fs (fs = sqrt(hbar w0 / kIUnit),
// so that |a|^2 is the intensity in kIUnit W/m^2) and the FP64 ADK constants K1, K3, K5 of both
// stages.
struct NLSetup {
    NLConst nl;          // nl.dz = 0: the caller sets the step length
    float sst_c_full;    // gamma2 / (w0 fs^2), the self-steepening factor when it is on
    int gas_ok;          // the gas is one of the seven of plasma.c
    double I1, I2;       // ionization potentials [eV]
    double K1[2], K3[2], K5[2];
};

inline NLSetup nl_setup(const mpc_params& p, double fs) {
    NLSetup s;
    memset(&s, 0, sizeof s);
    NLConst& n = s.nl;
    const double fs2 = fs * fs;
    n.gam = (float)(p.gamma2 / fs2);
    s.sst_c_full = (float)(p.gamma2 / (p.w0 * fs2));
    n.sst_c = p.sst_on == 1 ? s.sst_c_full : 0.0f;
    n.I_scale = (float)kIUnit;
    const double E_c = sqrt(2.0 * kZW0 / kNC) * kFCTR / kEF;  // plasma.c:145-149
    n.E_c = (float)E_c;
    n.inv_E_c = (float)(1.0 / E_c);
    double Natm = 0, sig = 0;
    s.gas_ok = gas_tables(p.gas, &s.I1, &s.I2, &Natm, &sig);
    const double Iion[2] = {s.I1 / kIH, s.I2 / kIH};
    const double nq[2] = {1.0 / sqrt(2.0 * Iion[0]), 2.0 / sqrt(2.0 * Iion[1])};
    for (int st = 0; st < 2; st++) {
        const double Cnl = sqrt(pow(2.0, 2.0 * nq[st]) / (nq[st] * tgamma(nq[st] + 1.0) * tgamma(nq[st])));
        s.K1[st] = Cnl * Cnl * sqrt(6.0 / M_PI) * 1.0 * Iion[st];
        s.K3[st] = 2.0 * pow(2.0 * Iion[st], 1.5);
        s.K5[st] = 2.0 * nq[st] - 0.0 - 1.5;
        n.l2K1[st] = (float)log2(s.K1[st]);
        n.l2K3[st] = (float)log2(s.K3[st]);
        n.K5[st] = (float)s.K5[st];
        n.K3l2e[st] = (float)(s.K3[st] / (3.0 * M_LN2));
    }
    const double Kon = p.deltat / kT0;
    n.Kon = (float)Kon;
    // v_e = sqrt(2 e^2 E0^2 / (4 me^2 w0^2)) with E0 = F EF (plasma.c:203, drift from w0 only)
    n.Kuv = (float)(sig * p.rho_nt * kEL0 * kEF / (sqrt(2.0) * kME * p.w0));
    const double k0ion = p.w0 / kC0;  // plasma.c:141
    n.K4w0 = (float)(k0ion / (p.n0 * p.rho_c) * p.w0 * p.w0);
    n.w0sq = (float)(p.w0 * p.w0);
    n.inv_w0 = (float)(1.0 / p.w0);
    n.invI1_Kon = s.I1 > 0 ? (float)(Kon / s.I1) : 0.0f;
    n.rho_half = (float)(p.rho_nt / 2.0);
    n.plasma = (p.plasm == 1) ? 1 : 0;
    return s;
}

}  // namespace mpc
