"""Electron-optics helpers of the simulator surface (host side).

Formulas follow namsa/optics.py: wavelength (:4-12), interaction parameter
(:100-108) and the Scherzer defocus (:69-72).
"""
from __future__ import annotations

import numpy as np
from scipy.constants import electron_mass, elementary_charge, speed_of_light


def voltage2Lambda(voltage):
    """Relativistic electron wavelength (Angstrom) for an accelerating voltage in V."""
    return 12.2643 / np.sqrt(voltage + 0.97845e-6 * voltage ** 2)


def sigma_int(voltage):
    """Interaction parameter sigma (rad / (V Angstrom)) for an accelerating voltage in V."""
    mc2 = electron_mass * speed_of_light ** 2
    ev = elementary_charge * voltage
    return 2 * np.pi * (mc2 + ev) / (2 * mc2 + ev) / (voltage2Lambda(voltage) * voltage)


def scherzer_defocus(Lambda, Cs):
    """Scherzer defocus sqrt(1.5 Cs lambda) (Angstrom)."""
    return np.sqrt(1.5) * np.sqrt(Cs * Lambda)
