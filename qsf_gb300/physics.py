"""Host-side pulses, fields and couplings, mirroring the reference's vocabulary.

These are per-step scalars evaluated on the host exactly as the reference does
(field_p.h, field.h, coupling.h); the GPU receives them as per-step coupling rows.

* ``Pulse``     -- _FieldConfig + PulsePrototype (field_p.h:6-12, 30-33) with the
                   pulse shapes SinPulse, Sin2Envelope<SinPulse>, ConstantPulse,
                   ChemPhysPulse (field_p.h:47-78, 100-116)
* ``Field``     -- Field<AXIS, Pulses...> (field.h:9-53)
* ``Coupling``  -- DipoleCoupling<VelocityGauge, Fields...> (coupling.h:101-118) with
                   PromoteFieldToA (field.h:103-133); in the length gauge the fields
                   are used as E(t) and couple x.E(t) in X space
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Sequence

PULSE_SIN, PULSE_SIN2_SIN, PULSE_CONST, PULSE_CHEMPHYS = 0, 1, 2, 3
GAUGE_VELOCITY, GAUGE_LENGTH = 0, 1
AXIS_X, AXIS_Y, AXIS_Z = 1, 2, 4
UNIT_INTENSITY = 3.50944e16  # W/cm^2 per atomic unit of intensity (constants.h:35)
LAMBDA2OMEGA = 45.563352529  # nm -> a.u. (constants.h:47-51)


def field_from_intensity(intensity_wcm2: float) -> float:
    """Peak field F0 = sqrt(I / 3.50944e16) in atomic units."""
    return math.sqrt(intensity_wcm2 / UNIT_INTENSITY)


def omega_from_wavelength(nm: float) -> float:
    return LAMBDA2OMEGA / nm


@dataclass
class Pulse:
    field: float
    omega: float
    ncycles: float
    phase_in_pi_units: float = 0.0
    delay_in_cycles: float = 0.0
    FWHM_percent: float = 0.0
    shape: int = PULSE_SIN2_SIN

    @property
    def phi(self) -> float:
        return self.phase_in_pi_units * math.pi

    @property
    def pulse_time(self) -> float:
        return 2.0 * math.pi * self.ncycles / self.omega

    def __call__(self, time: float) -> float:
        if self.shape == PULSE_SIN:
            return self.field * math.sin(self.omega * time + self.phi)
        if self.shape == PULSE_SIN2_SIN:
            env_mult = self.omega / (2.0 * self.ncycles)
            s = math.sin(env_mult * time)
            return self.field * math.sin(self.omega * time + self.phi) * (s * s)
        if self.shape == PULSE_CONST:
            return self.field
        if self.shape == PULSE_CHEMPHYS:
            env_mult = self.omega / (2.0 * self.ncycles)
            tmp = self.omega * time + self.phi - math.pi * self.ncycles
            return self.field * (math.sin(env_mult * time) * math.cos(tmp) +
                                 math.cos(env_mult * time) * math.sin(tmp) / self.ncycles)
        raise ValueError("unknown pulse shape")


@dataclass
class Field:
    axis: int
    pulses: List[Pulse]

    def delay(self, p: Pulse) -> float:
        return p.delay_in_cycles * 2.0 * math.pi / p.omega

    def end(self, p: Pulse) -> float:
        return self.delay(p) + p.pulse_time

    def __call__(self, time: float) -> float:
        val = 0.0
        for p in self.pulses:
            d, e = self.delay(p), self.end(p)
            val += p(time - d) if not (time > e or time < d) else 0.0
        return val

    def max_duration(self) -> float:
        mx = self.end(self.pulses[0]) if self.pulses else 0.0
        for p in self.pulses:
            mx = max(mx, self.end(p))
        return mx


class Coupling:
    """Coupling state across steps (PromoteFieldToA keeps A and the previous time)."""

    def __init__(self, gauge: int, fields: Sequence[Field] = ()):
        self.gauge = gauge
        self.fields = list(fields)
        self.last = [0.0] * len(self.fields)
        self.prev_time = [0.0] * len(self.fields)

    @property
    def size(self) -> int:
        return len(self.fields)

    @property
    def couples_in_x(self) -> bool:
        return self.gauge == GAUGE_LENGTH

    def max_pulse_duration(self) -> float:
        m = 0.0
        for f in self.fields:
            m = max(m, f.max_duration())
        return m

    def precalc(self, time: float) -> None:
        for i, f in enumerate(self.fields):
            F = f(time)
            if self.gauge == GAUGE_VELOCITY:
                prev = self.last[i]
                self.last[i] = prev + (self.prev_time[i] - time) * F
                self.prev_time[i] = time
            else:
                self.last[i] = F

    def vector(self) -> List[float]:
        out = []
        for d in range(3):
            s = 0.0
            first = True
            for f, v in zip(self.fields, self.last):
                term = v if (f.axis >> d) & 1 else 0.0
                s = term if first else s + term
                first = False
            out.append(s)
        return out
