"""Piecewise parsing of .in files, and the parallel CSR fill, give the same
result as one pass.

SMG_IO_PIECE_BYTES shrinks the loader's pieces to a few bytes, so small
random files, with any whitespace between tokens, records split across
lines, CRLF endings and planted errors, are cut at many record boundaries.
Status, and for valid files the CSR, must equal the single-piece read."""
import os

import numpy as np
import pytest

from clustersm_gb300.native import HostGraph, SmgError

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")
given, settings = hyp.given, hyp.settings


def _read(path, piece):
    """Read with pieces of `piece` bytes and the parallel CSR fill forced on
    (piece 0: one piece, one-thread fill)."""
    keys = ("SMG_IO_PIECE_BYTES", "SMG_IO_SCATTER_MIN")
    old = {k: os.environ.get(k) for k in keys}
    if piece:
        os.environ["SMG_IO_PIECE_BYTES"] = str(piece)
        os.environ["SMG_IO_SCATTER_MIN"] = "0"
    else:
        for k in keys:
            os.environ.pop(k, None)
    try:
        g = HostGraph.read(path)
        return 0, (g.offsets().tolist(), g.neighbors().tolist(), g.labels().tolist())
    except SmgError as e:
        return e.status, None
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


@st.composite
def in_files(draw):
    n = draw(st.integers(1, 12))
    pairs = [(a, b) for a in range(n) for b in range(a + 1, n)]
    chosen = draw(st.lists(st.sampled_from(pairs), unique=True, max_size=len(pairs))) if pairs else []
    edges = [(b, a) if draw(st.booleans()) else (a, b) for a, b in chosen]
    labels = draw(st.lists(st.integers(0, 5), min_size=n, max_size=n))
    deg = [0] * n
    for a, b in edges:
        deg[a] += 1
        deg[b] += 1
    order = draw(st.permutations(range(n)))
    recs = [["t", str(n), str(len(edges))]]
    recs += [["v", str(v), str(labels[v]), str(deg[v])] for v in order]
    recs += [["e", str(a), str(b)] for a, b in edges]
    # planted errors (the file must then be rejected either way)
    bad = draw(st.sampled_from(["none", "none", "none", "short", "type", "range", "twice", "degree", "count"]))
    if bad == "short" and len(recs) > 1:
        i = draw(st.integers(1, len(recs) - 1))
        recs[i] = recs[i][:-1]
    elif bad == "type" and len(recs) > 1:
        recs[draw(st.integers(1, len(recs) - 1))][0] = "x"
    elif bad == "range" and edges:
        recs[-1][2] = str(n)
    elif bad == "twice":
        recs.insert(draw(st.integers(1, len(recs))), list(recs[1]))
    elif bad == "degree":
        recs[1][3] = str(int(recs[1][3]) + 1)
    elif bad == "count":
        recs[0][2] = str(len(edges) + 1)
    seps = st.sampled_from([" ", "  ", "\t", "\n", "\r\n", " \n"])
    ends = st.sampled_from(["\n", "\r\n", "\n\n", " \n"])
    out = []
    for r in recs:
        out.append(draw(seps).join(r) if len(r) > 1 else r[0])
        out.append(draw(ends))
    if draw(st.booleans()):
        out.pop()  # no final line end
    return "".join(out)


@settings(max_examples=300, deadline=None)
@given(text=in_files(), piece=st.integers(1, 24))
def test_pieces_match_single_pass(tmp_path_factory, text, piece):
    p = tmp_path_factory.mktemp("pieces") / "g.in"
    p.write_text(text, newline="")
    one = _read(p, 0)
    many = _read(p, piece)
    assert one == many, (text, piece)
