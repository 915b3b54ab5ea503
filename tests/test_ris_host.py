"""CPU: the host side of the dense RIS fill (solver_gb300/ris.py), no GPU touched.

* voxel_bodies (the benchmark's RIS bodies of a voxel mesh) describes the same bricks and
  faces as the tests' own construction (tests/ris_cases.py), which the fill parity tests
  use;
* the body arrays are accepted in the reference's layouts: the (count, width) matrix, the
  JSON's width lists of count values, symbol- or string-keyed dicts; wrong shapes are
  refused before any call into the library."""
import numpy as np
import pytest

from solver_gb300 import configs, ris
from tests import ris_cases


def test_voxel_bodies_match_the_test_construction():
    c = ris_cases.voxel_case(configs.crossbar_20x20x4())
    v1, s1 = ris_cases.ris_geometry(c)
    cell = (c["cc"]["sx"], c["cc"]["sy"], c["cc"]["sz"])
    v2, s2 = ris.voxel_bodies(c["inc"], c["exp"], c["grid"], cell)
    scale = max(cell)
    assert np.max(np.abs(v1["coordinate"] - v2["coordinate"])) <= 1e-12 * scale
    assert np.array_equal(v1["S"], v2["S"])
    assert np.max(np.abs(v1["centri"] - v2["centri"])) <= 1e-12 * scale
    corners = [0, 1, 2, 9, 10, 11]  # the two vertices calcola_P reads
    assert np.max(np.abs(s1["estremi_celle"][:, corners] - s2["estremi_celle"][:, corners])) \
        <= 1e-12 * scale
    assert np.array_equal(s1["S"], s2["S"])


def test_body_arrays_take_the_reference_layouts():
    vol, surf = ris_cases.random_bodies(5, 4, 3, 2, 6)
    m, ns = 9, 6
    a = ris.ris_volumes(vol, m)
    # the JSON layout: 24 lists of m values; symbol keys as the reference's volumi has them
    b = ris.ris_volumes({":coordinate": vol["coordinate"].T.tolist(), ":S": list(vol["S"]),
                         ":centri": np.asarray(vol["centri"]).T}, m)
    for k in ("coordinate", "S", "centri"):
        assert np.array_equal(a[k], b[k])
        assert a[k].flags["C_CONTIGUOUS"]
    c = ris.ris_surfaces({"estremi_celle": surf["estremi_celle"].T, "S": surf["S"],
                          "centri": surf["centri"]}, ns)
    assert np.array_equal(c["estremi_celle"], np.asarray(surf["estremi_celle"]))
    # centres are optional (read only for the retarded operator)
    assert not ris.ris_surfaces({"estremi_celle": surf["estremi_celle"], "S": surf["S"]},
                                ns)["centri"].any()
    with pytest.raises(ValueError, match="coordinate"):
        ris.ris_volumes({"coordinate": np.zeros((m, 23)), "S": np.ones(m)}, m)
    with pytest.raises(ValueError, match="S must have"):
        ris.ris_surfaces({"estremi_celle": surf["estremi_celle"], "S": np.ones(ns + 1)}, ns)


def test_ports_map_to_the_nearest_node():
    """find_nodes_ports_or_le: positions rounded to 5 decimals, scaled, then the first node
    at the smallest distance (ties to the lower index)."""
    nodes = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [1.0, 0.0, 0.0]])
    ports = [{"inputElement": [0.9, 0.1, 0.0], "outputElement": [0.1, 0.8, 0.0]},
             {"inputElement": [0.000004, 0.0, 0.0], "outputElement": [2.0, 0.0, 0.0]}]
    les = [{"inputElement": [0.0, 0.0, 0.0], "outputElement": [0.0, 1.0, 0.0], "type": 1,
            "rlcParams": {"resistance": 50.0}}]
    p, le = ris.find_nodes_ports_or_le(ports, les, nodes, 1.0)
    # node 3 duplicates node 1: the first one wins
    assert p["port_nodes"].tolist() == [[1, 2], [0, 1]]
    assert le["le_nodes"].tolist() == [[0, 2]] and le["R"] == [50.0] and le["L"] == [0.0]
    # rounding to 5 decimals before scaling: 0.000004 m rounds to 0
    assert p["port_start"][1][0] == 0.0
    # the JSON layout of the node coordinates (three lists) and a unit scale
    p2, _ = ris.find_nodes_ports_or_le(ports, [], nodes.T, 1.0)
    assert np.array_equal(p2["port_nodes"], p["port_nodes"])
    p3, _ = ris.find_nodes_ports_or_le([{"inputElement": [900.0, 100.0, 0.0],
                                         "outputElement": [0.0, 0.0, 0.0]}], [], nodes, 1e-3)
    assert p3["port_nodes"].tolist() == [[1, 0]]


def test_z_self_reads_symbol_keyed_volumi():
    rng = np.random.default_rng(4)
    vol = {"R": rng.uniform(0, 1, 10), "Cd": rng.uniform(1e-12, 2e-12, 10),
           "indici_dielettrici": np.array([2, 5]), "Zs_part": rng.uniform(0, 1e-6, 10)}
    sym = {":" + k: v for k, v in vol.items()}
    w = 2 * np.pi * 1e9
    for zs in (False, True):
        assert np.array_equal(ris.z_self(vol, w, zs), ris.z_self(sym, w, zs))
