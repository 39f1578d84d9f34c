"""Writes the golden fixtures of tests/golden/ from the CPU oracle (FP64).

The reference ships no numeric golden vectors and cannot run here (Julia), so these fixtures are
oracle outputs on seeded inputs, committed so that GPU parity can be checked without recomputing
the oracle and so that any drift in the oracle itself is caught. Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402
from fields import curl_noise_3d, e_config1, e_config2, solenoidal_2d, spectrum_field  # noqa: E402


def main():
    out = {}
    u, ks = spectrum_field((64, 64), e_config1, seed=1)
    c, T, P = O.spectral_flux(u, ks, ("linear", 1.0), "two_thirds")
    _, _, _, sidx = O.shell_setup(ks, ("linear", 1.0))
    out["flux64_u"], out["flux64_T"], out["flux64_P"], out["flux64_centers"], out["flux64_sidx"] = u, T, P, c, sidx
    u3, ks3 = spectrum_field((16, 16, 16), e_config2, seed=3)
    for d in ("two_thirds", "three_halves"):
        _, e, T3, net, asym = O.shell_to_shell(u3, ks3, ("linear", 2.0), d)
        out[f"s2s16_{d}_T"], out[f"s2s16_{d}_net"] = T3, net
    out["s2s16_u"], out["s2s16_edges"] = u3, e
    un, ksn = curl_noise_3d(12, 7)
    out["nl12_u"] = un
    for d in ("none", "two_thirds", "three_halves"):
        out[f"nl12_{d}_N"] = O.nonlinear_term(un, ksn, d)
    chans, _, _ = O.partial_fluxes(un, ksn, "helical", ("linear", 1.0), "two_thirds")
    out["pf12_T"] = np.stack([chans[(a, b, c)][0] for a in ("positive", "negative") for b in ("positive", "negative")
                              for c in ("positive", "negative")])
    u2, ks2 = solenoidal_2d(12, 21)
    net2, S2 = O.mode_to_mode_triad(u2, ks2, "two_thirds")
    out["m2m12_u"], out["m2m12_S"], out["m2m12_net"] = u2, S2, net2
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
