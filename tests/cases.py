"""Known-answer cases shared by the CPU (oracle) and GPU tests."""

import json
import os

import numpy as np

from galacticus_gb300 import _abi, workloads

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def known_answers():
    with open(os.path.join(GOLDEN, "reference_known_answers.json")) as f:
        return json.load(f)


def box_case():
    """closedBox and leakyBox (testSuite/parameters/reproducibility/
    {closedBox,leakyBox}.xml with {closedBox,leakyBox}Tree.xml): one node of
    1e12 Msun from t=12.47 to 13.47 Gyr with a 1e11 Msun gaseous disk, a
    fixed star-formation timescale, R=0.4, p=0.025, tolerances 1e-6 / 1e-3;
    leakyBox adds a fixed outflow fraction of 1 under a rate limit of 1e-3."""
    ka = known_answers()
    cases = {}
    for name in ("closedBox", "leakyBox"):
        case = ka[name]
        p = _abi.default_params()
        p.ode_tolerance_absolute = 1.0e-6
        p.ode_tolerance_relative = 1.0e-3
        p.physics = _abi.PHYS_STAR_FORMATION_DISK
        p.sf_disk.timescale_type = _abi.SF_TIMESCALE_FIXED
        p.sf_disk.timescale_fixed = case["timescale"]
        p.recycled_fraction = 0.4
        p.metal_yield = 0.025
        if name == "leakyBox":
            p.physics |= _abi.PHYS_FEEDBACK_DISK
            p.outflow_disk.type = _abi.OUTFLOW_FIXED
            p.outflow_disk.fraction = 1.0
            p.outflow_disk.timescale_fractional_minimum = 1.0e-3
        state = np.zeros((_abi.NY, 1))
        state[_abi.Y_DISK_GAS] = 1.0e11
        cosmo = workloads.Cosmology(omega_matter=0.3, omega_lambda=0.7, omega_baryon=0.05, hubble=70.0)
        r, v = cosmo.virial(np.array([1.0e12]), cosmo.redshift(np.array([12.47])))
        param = np.zeros((_abi.NP, 1))
        param[:, 0] = [1.0e12, 0.0, r[0], v[0], 0.05]
        batch = workloads.Batch(state, param, np.array([12.47]), np.array([13.47]), np.array([-1.0]))
        expect = [case["diskMassGas"], case["diskMassStellar"], case["diskAbundancesGasMetals"],
                  case["diskAbundancesStellarMetals"]]
        cases[name] = (p, batch, expect, case["toleranceRelative"])
    return cases
