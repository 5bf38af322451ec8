"""Moving-domain scenarios with stochastic species, shared by the CPU and GPU
tests of the coupled flow + NSM path."""
import numpy as np

from spatialpy_gb300 import scenario as S


def dam_break_species(spacing_div=16, num_steps=60, num_outputs=4, D=0.05, molecules=2000,
                      network="decay", dims=3):
    """The dam break (fluid type 1, walls type 2) with one species S diffusing
    in the fluid only.  network: "decay" (S -> 0), "full" (adds 0 -> S on
    fluid particles, whose rate k*vol follows the changing density, and
    2S -> 0, whose rate uses 1/vol), "none" (diffusion only).  dims=2: the
    dam break in the xy-plane."""
    sc = S.config_dam_break(spacing_div=spacing_div, num_steps=num_steps,
                            num_outputs=num_outputs, species_D=D, molecules=molecules,
                            dims=dims)
    rxns = {"decay": [(0.01, {"S": 1}, {}, None)],
            "full": [(0.5, {"S": 1}, {}, None), (2e5, {}, {"S": 1}, [1]),
                     (2e-7, {"S": 2}, {}, None)],
            "none": []}[network]
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(["S"], rxns, 2)
    return sc.copy(rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac.reshape(-1, 2),
                   rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN,
                   name=f"dam_break_species_{network}")


def dam_break_chem(spacing_div=8, num_steps=41, num_outputs=4, D=0.05, molecules=2000):
    """The dam break with deterministic chemistry (Model.enable_pde): one
    species S diffusing in the fluid and decaying (k 0.01), concentrations
    starting at the scattered counts.  With one species and one reaction the
    reference's transposed reads of the diffusion matrix and the
    stoichiometry (model.cpp:165, 186) agree with their layouts, so the
    compiled engine can be compared on it."""
    sc = S.config_dam_break(spacing_div=spacing_div, num_steps=num_steps,
                            num_outputs=num_outputs, species_D=D, molecules=molecules)
    programs = {}
    rate, kind, reac, allowed, jcN, irN, prN = S.mass_action(
        ["S"], [(0.01, {"S": 1}, {}, None)], 2, {}, [], programs)
    return sc.copy(rxn_rate=rate, rxn_kind=kind, rxn_reactants=reac.reshape(-1, 2),
                   rxn_allowed=allowed, jcN=jcN, irN=irN, prN=prN, enable_pde=True,
                   name="dam_break_chem", **programs)
