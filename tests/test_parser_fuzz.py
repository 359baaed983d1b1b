"""The engine's parser (csg_tree_parse) and the oracle's against the reference's own
CSGTree::Parse (CSGRayCasting/Graphics/RayCasting/CSGTree/CSGTree.cu:5-200, compiled for
the host under oracle/_ref) on seeded mutations of valid scene texts: odd numbers (nan,
inf, hex floats, overflow, underflow, numeric prefixes), odd colours (signs, 0x prefixes,
multi-byte characters), swapped, deleted, inserted and misspelt keywords, and unusual
separators.  Where the reference parses, the nodes and primitives must be the same bytes;
where it throws, the message must be the same text.

The reference reads past the end of its token list when a primitive is cut short
(CSGTree.cu:61-131, undefined behaviour): such texts are never given to it; the engine and
the oracle must reject them.  The reference's host build exists only where its sources do,
so the test is skipped elsewhere."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

OPS = (b"Union", b"Difference", b"Intersection")
ARITY = {b"Sphere": 5, b"Cube": 5, b"Cylinder": 9}
SPACES = b" \t\n\r\x0b\x0c"

NUMBERS = [b"nan", b"-nan", b"NAN", b"nan(12)", b"inf", b"-inf", b"Infinity", b"1e50", b"-1e50",
           b"1e-50", b"1e-39", b"-1e-39", b"1.2e-38", b"3.4028235e38", b"3.40282357e38", b"3.4028236e38",
           b"1e39", b"0x1p3", b"0x1.8p1", b"0x", b"0X10", b"abc", b"1.5abc", b"-0", b"+3", b".5", b"5.",
           b"1e", b"e5", b"-", b"+", b"0", b"360", b"361", b"360.0000000001", b"-1e-300", b"1e400",
           b"1e-400", b"1,5", b"0.0000001", b"12345678901234567890", b"\xd9\xa3", b"1\x002"]
COLOURS = [b"GG0000", b"-1FFFF", b"+FFFFF", b"0x0000", b"0X12ab", b"FFFFF", b"FFFFFFF", b"ffFFff",
           b"-00000", b"+-0000", b"1e5FFF", b"\xc3\x84\xc3\x960", b"\xff\xfe0000", b"00\x00000",
           b"g00000", b"0xFF00", b"7FFFFF", b"000000"]
WORDS = [b"Union", b"Difference", b"Intersection", b"Sphere", b"Cube", b"Cylinder", b"union",
         b"SPHERE", b"Spheres", b"Cub", b"Union\x00", b"#", b"1", b"FF0000"]


def _tokens(text: bytes) -> list[bytes]:
    return text.split()  # ASCII whitespace: the classic-locale set `ss >> str` splits on


def reads_past_end(toks: list[bytes]) -> bool:
    """True when the reference's token walk reaches a primitive whose parameters run past
    the end of the list.  The walk ignores every other error, so it errs on the side of
    keeping texts away from the reference."""
    i = 0
    while i < len(toks):
        t = toks[i]
        if t in OPS:
            i += 1
            continue
        need = ARITY.get(t)
        if need is None:
            return False  # the reference throws "Unrecognized keyword" here
        if i + need >= len(toks):
            return True
        i += need + 1
    return False


def _mutate(rng, text: bytes) -> bytes:
    toks = _tokens(text)
    for _ in range(int(rng.integers(1, 4))):
        if not toks:
            toks = [WORDS[int(rng.integers(len(WORDS)))]]
        k = int(rng.integers(len(toks)))
        kind = int(rng.integers(10))
        if kind <= 2:  # a number slot (anything that is not a keyword or a colour)
            slots = [j for j, t in enumerate(toks) if t not in OPS and t not in ARITY and len(t) != 6]
            if slots:
                toks[slots[int(rng.integers(len(slots)))]] = NUMBERS[int(rng.integers(len(NUMBERS)))]
        elif kind == 3:  # a colour slot
            slots = [j for j, t in enumerate(toks) if len(t) == 6 and t not in OPS]
            if slots:
                toks[slots[int(rng.integers(len(slots)))]] = COLOURS[int(rng.integers(len(COLOURS)))]
        elif kind == 4:
            toks[k] = WORDS[int(rng.integers(len(WORDS)))]
        elif kind == 5:
            del toks[k]
        elif kind == 6:
            toks.insert(k, WORDS[int(rng.integers(len(WORDS)))])
        elif kind == 7 and k + 1 < len(toks):
            toks[k], toks[k + 1] = toks[k + 1], toks[k]
        elif kind == 8:
            toks = toks[:k]
        else:
            toks.insert(k, toks[k])
    seps = [bytes([SPACES[int(rng.integers(len(SPACES)))]]) for _ in range(len(toks))]
    out = b"".join(t + s for t, s in zip(toks, seps))
    if rng.random() < 0.2:
        out = b"\xa0" * int(rng.integers(0, 2)) + out  # not a separator in the classic locale
    return out


def _base_texts():
    from csgrt import scenes
    texts = [scenes.write_text(scenes.wikipedia_tree()).encode()]
    texts += [scenes.write_text(scenes.random_tree(s, 2, 6, 4)).encode() for s in range(10)]
    for f in sorted((GOLDEN / "scenes").glob("*.txt"))[:8]:
        data = f.read_bytes()
        if len(data) < 4000:
            texts.append(data)
    return texts


def _ref_prims_defined(nodes, prims):
    """The reference leaves a sphere's or cube's unused parameter slots uninitialised;
    the engine and the oracle write zeros there."""
    p = prims.copy()
    for i in range(len(nodes)):
        if nodes["prim"][i] >= 0 and nodes["type"][i] != 4:
            p["p"][nodes["prim"][i], 1:] = 0
    return p


def test_parser_matches_reference_on_mutated_texts(csg, oracle):
    from oracle import ParseError, RefHost
    if not RefHost.available():
        pytest.skip("the reference's host build is not present here")
    ref = RefHost()
    rng = np.random.default_rng(20261204)
    bases = _base_texts()
    outcomes = {"ok": 0, "error": 0, "past_end": 0}
    messages = set()
    for case in range(3000):
        text = _mutate(rng, bases[case % len(bases)])
        if reads_past_end(_tokens(text)):
            outcomes["past_end"] += 1
            with pytest.raises(csg.CsgError):
                csg.parse_tree(text)
            with pytest.raises(ParseError):
                oracle.parse(text)
            continue
        try:
            rn, rp = ref.parse(text)
        except ParseError as e:
            outcomes["error"] += 1
            messages.add(e.msg)
            with pytest.raises(csg.CsgError) as ce:
                csg.parse_tree(text)
            assert ce.value.msg == e.msg, (case, text)
            with pytest.raises(ParseError) as oe:
                oracle.parse(text)
            assert oe.value.msg == e.msg, (case, text)
            continue
        outcomes["ok"] += 1
        en, ep, _ = csg.parse_tree(text)
        rp = _ref_prims_defined(rn, rp)
        assert (en == rn.view(np.uint8).ravel()).all(), (case, text)
        assert (ep == rp.view(np.uint8).ravel()).all(), (case, text)
        on, op = oracle.parse(text)
        assert (on.view(np.uint8) == rn.view(np.uint8)).all(), (case, text)
        assert (op.view(np.uint8) == rp.view(np.uint8)).all(), (case, text)
    # the mutations reach every outcome and many distinct errors
    assert outcomes["ok"] >= 300 and outcomes["error"] >= 1000 and outcomes["past_end"] >= 100, outcomes
    assert len(messages) >= 8, messages


def test_past_end_walk():
    assert reads_past_end(_tokens(b"Union Sphere 0 0 0 FF0000 1 Sphere 1 0"))
    assert reads_past_end(_tokens(b"Cylinder 0 0 0 FF0000 1 2 0 0"))
    assert not reads_past_end(_tokens(b"Union Sphere 0 0 0 FF0000 1 Sphere 1 0 0 00FF00 1"))
    assert not reads_past_end(_tokens(b"Union Spere 0 0 0 FF0000 1 Sphere 1 0"))
