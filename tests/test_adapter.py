"""The product's C++ adapter (flexaidds_gb300/adapter/): compiled against the reference's own
headers (oracle/Makefile, target ref), its packing of the reference's set-up state into the C ABI's
descriptors is compared byte for byte with the descriptors the reference's set-up exported into the
golden fixtures. The adapter's backend (fxe_flexaid_backend.cpp: fxe_context_create, fxe_eval_ic)
is compiled there too. Needs the reference checkout (skipped without it)."""
import os

import numpy as np
import pytest

from oracle import ref

pytestmark = pytest.mark.skipif(not os.path.exists(ref.LIB_PATH),
                                reason="oracle/_ref not built (needs the reference checkout)")

NAMES = ["c0_2000_24", "curves_900_16", "outside_600_10", "scale_6000_48", "flex_2000_24", "flexcurves_900_16"]


@pytest.mark.parametrize("name", NAMES)
def test_adapter_packs_the_reference_setup(name):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from conftest import load_golden
    import test_host
    d, _ = load_golden(name)
    inp = test_host._make_golden().inputs_for(name)
    h = ref.RefHarness(inp)
    a = h.adapter_arrays()

    def same(x, y, k):
        x, y = np.ascontiguousarray(x).reshape(-1), np.ascontiguousarray(y).reshape(-1)
        assert x.dtype == y.dtype, (k, x.dtype, y.dtype)
        assert x.tobytes() == y.tobytes(), k

    for k in ("rec_xyz", "rec_radius", "rec_type", "grid_ic", "lig_radius", "lig_type", "lig_rec", "lig_shift",
              "lig_ic", "build_order", "bonded", "gene_typ", "gene_atm", "gene_min", "gene_max", "gene_del",
              "gene_map", "emat_weight", "emat_off", "emat_x", "emat_y"):
        same(a[k], getattr(d, k), k)
    f = a["frame"]
    same(f[0:3], d.ori, "ori")
    same(f[3:6], d.globalmin, "globalmin")
    same(f[6:9], d.globalmax, "globalmax")
    assert f[9] == np.float32(d.maxwidth)
    assert tuple(a["params"]) == (np.float32(d.permeability), np.float32(d.dee_clash), float(d.intramolecular),
                                  np.float32(d.solventterm))
    if d.n_flex:
        info = a["flex_info"].reshape(-1, 4)
        same(info[:, 0], d.flex_first, "flex_first")
        same(info[:, 1], d.flex_natm, "flex_natm")
        same(info[:, 2], d.flex_nrot, "flex_nrot")
        same(a["flex_backbone"], d.flex_isbb, "flex_isbb")
        same(a["flex_xyz"], d.flex_xyz, "flex_xyz")
        same(a["flex_bonded"], d.flex_bonded, "flex_bonded")
