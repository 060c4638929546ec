// components.h -- slot layout of the wave-component tables that the host
// forms for the spectral wavemakers and the kernels read (S.jon, slot-major
// [kJonSlots][n]).
#pragma once

namespace nhw {

// LEF_JON / LEF_TMA / LEF_SPC: wave height Wh, angular frequency, wave
// number, Stokes drift, phase, sinh(k h), sin and cos of the direction
constexpr int kJonSlots = 8;
constexpr int kJonPhase = 4;
// The internal makers INT_JON / INT_TMA / INT_SPC / INT_IRR: Celerity *
// Amp_Wave (2 Celerity for INT_IRR's first frequency), Amp_Wave / 2 (that
// component only), Segma, the cross-channel wave number WnumY, the phase
// (kJonPhase) and the kind (1: INT_IRR's first frequency, 0: the rest)
constexpr int kIntPre = 0, kIntHalfAmp = 1, kIntSegma = 2, kIntWnumY = 3, kIntKind = 5;

}  // namespace nhw
