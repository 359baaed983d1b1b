"""The engine's scene parser (csg_tree_parse) against the reference parser's golden
output and error messages, and against the oracle on generated scenes."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN


def test_parse_reference_scene_files_bit_exact(csg):
    data = np.load(GOLDEN / "ref_parse.npz")
    for f in sorted((GOLDEN / "scenes").glob("*.txt")):
        nodes, prims, depth = csg.parse_tree(f.read_bytes())
        assert (nodes == data[f"{f.stem}/nodes"].ravel()).all(), f.stem
        assert (prims == data[f"{f.stem}/prims"].ravel()).all(), f.stem
        assert depth >= 0


def test_parse_errors_match_reference_messages(csg):
    cases = json.loads((GOLDEN / "ref_errors.json").read_text())
    assert len(cases) >= 15
    for c in cases:
        if c["ok"]:
            nodes, prims, _ = csg.parse_tree(c["text"])
            assert len(nodes) // 44 == c["nodes"]
        else:
            with pytest.raises(csg.CsgError) as e:
                csg.parse_tree(c["text"])
            assert e.value.msg == c["message"], c["text"]
            assert e.value.code in (csg.CSG_E_PARSE, csg.CSG_E_RANGE, csg.CSG_E_COUNT)


def test_parse_error_codes(csg):
    codes = {
        "Union Cylinder 0 0 0 FF0000 1 2 361 0 0 Sphere 1 0 0 00FF00 1": csg.CSG_E_RANGE,
        "Union Sphere 0 0 0 FF0000 1e50 Sphere 1 0 0 00FF00 1": csg.CSG_E_RANGE,
        "Union Sphere 0 0 0 FF0000 1": csg.CSG_E_COUNT,
        "Spere 0 0 0 FF0000 1": csg.CSG_E_PARSE,
        # a primitive cut short at the end of the text (undefined behaviour in the
        # reference, which indexes past its token list)
        "Union Sphere 0 0 0 FF0000 1 Sphere 1 0": csg.CSG_E_PARSE,
        "Cylinder 0 0 0 FF0000 1 2 0 0": csg.CSG_E_PARSE,
    }
    for text, code in codes.items():
        with pytest.raises(csg.CsgError) as e:
            csg.parse_tree(text)
        assert e.value.code == code, text


def test_parse_generated_scenes_match_oracle(csg, oracle):
    from csgrt import scenes
    texts = [scenes.write_text(scenes.wikipedia_tree())]
    texts += [scenes.write_text(scenes.cheese_tree(s)) for s in range(3)]
    texts += [scenes.write_text(scenes.random_tree(s)) for s in range(12)]
    for text in texts:
        nodes, prims, depth = csg.parse_tree(text)
        on, op = oracle.parse(text)
        assert (nodes == on.view(np.uint8).ravel()).all()
        assert (prims == op.view(np.uint8).ravel()).all()
        assert depth <= 12


def test_parse_whitespace_and_tokens(csg):
    a = csg.parse_tree("Union\n\tSphere 0 0 0 FF0000 1\n\tSphere 1 0 0 00ff00 1")
    b = csg.parse_tree("Union Sphere 0 0 0 FF0000 1\r\n\v\fSphere 1 0 0 00ff00 1   ")
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
    # std::stof parses a numeric prefix ("1.5abc" -> 1.5), as the reference does
    n, p, _ = csg.parse_tree("Cube 1.5abc 0 0 FF0000 2")
    assert np.frombuffer(p.tobytes()[4:8], np.float32)[0] == np.float32(1.5)


def test_primitive_limit(csg):
    from csgrt import scenes
    leaves = [("Sphere", 0, 0, 0, "FFFFFF", 0.1)] * 32768
    tree = scenes._balanced(leaves)
    with pytest.raises(csg.CsgError) as e:
        csg.parse_tree(scenes.write_text(tree))
    assert e.value.code == csg.CSG_E_DEPTH
