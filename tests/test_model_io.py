"""The native model file (format 1.4) against the reference's codec.

* Bytes written for a model equal the reference's SerializeModel bytes for the same
  trees, schema and objective (src/io/model_format.cpp, model_payload.cpp); the
  reference reads the files written here and the files it writes read here.
* The committed golden files (written by the reference, tests/golden/make_golden.py)
  read and rewrite byte for byte where the reference sources are absent.
* Malformed files fail as in the reference: integrity, version, kind, length,
  truncation, trailing bytes, reserved bytes, non-finite values, tree structure, split
  ranges and schema checks; files of minor versions 1 and 3 read like the reference.
No GPU is needed: the model codec is host code of the library.
"""

from __future__ import annotations

import json
import os
import struct

import numpy as np
import pytest

import mpsboost_gb300 as mb
from mpsboost_gb300._lib import NODE_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
OBJ = {"squared_error": 0, "binary_logistic": 1, "quantile": 2, "poisson": 3, "tweedie": 4}


def _fnv(b: bytes) -> int:
    h = 14695981039346656037
    for c in b:
        h = ((h ^ c) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def _refresh(data: bytes, payload: bytes | None = None) -> bytes:
    """Header with the payload's length and checksum (for hand-edited payloads)."""
    payload = data[32:] if payload is None else payload
    return data[:16] + struct.pack("<QQ", len(payload), _fnv(payload)) + payload


def _data(seed, rows=300, feats=4, nan=0.05):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(rows, feats)).astype(np.float32)
    x[rng.random(x.shape) < nan] = np.nan
    y = np.nan_to_num(x[:, 0]) * 2 + rng.normal(size=rows) * 0.1
    return x, y, rng.uniform(0.5, 1.5, rows)


CASES = [
    dict(objective="squared_error", params=dict(n_estimators=3, learning_rate=0.3, max_depth=3)),
    dict(objective="quantile", params=dict(n_estimators=2, learning_rate=0.5, max_depth=2, objective_alpha=0.7)),
    dict(objective="poisson", params=dict(n_estimators=2, learning_rate=0.2, max_depth=3)),
    dict(objective="tweedie", params=dict(n_estimators=2, learning_rate=0.2, max_depth=3,
                                          tweedie_variance_power=1.3)),
    dict(objective="binary_logistic", params=dict(n_estimators=2, learning_rate=0.3, max_depth=3)),
]


def _labels(objective, y):
    if objective == "binary_logistic":
        return (y > np.median(y)).astype(np.float64)
    if objective in ("poisson", "tweedie"):
        return np.abs(y)
    return y


@pytest.mark.parametrize("case", range(len(CASES)))
def test_bytes_equal_reference(reference, case):
    c = CASES[case]
    x, y, w = _data(30 + case)
    y = _labels(c["objective"], y)
    ds = reference.quantize_dense(x, 32)
    params = dict(c["params"], objective=c["objective"])
    model = reference.train_regressor(ds, y, w, **params)
    want = reference.model_to_bytes(model)
    ours = mb.RegressionModel(model.base_score, params["learning_rate"], model.trees,
                              objective=OBJ[c["objective"]],
                              objective_alpha=params.get("objective_alpha", 0.5),
                              tweedie_variance_power=params.get("tweedie_variance_power", 1.5))
    got = ours.to_bytes(ds)
    assert got == want
    # each side reads the other's files
    back = mb.RegressionModel.from_bytes(want)
    assert back.base_score == model.base_score and back.learning_rate == params["learning_rate"]
    assert back.objective == OBJ[c["objective"]]
    for t1, t2 in zip(back.trees, model.trees):
        assert t1.tobytes() == np.ascontiguousarray(t2, NODE_DTYPE).tobytes()
    assert np.array_equal(back.schema["boundaries"], ds.boundaries_flat)
    assert np.array_equal(back.schema["missing_counts"], ds.missing_counts)
    theirs = reference.model_from_bytes(got)
    for t1, t2 in zip(theirs.trees, model.trees):
        assert t1.tobytes() == t2.tobytes()


def _golden_files():
    with open(os.path.join(HERE, "golden", "reference_cases.json")) as fh:
        return [bytes.fromhex(c["model_file"]) for c in json.load(fh)["cases"]]


@pytest.mark.parametrize("index", range(8))
def test_golden_files_round_trip(index):
    data = _golden_files()[index]
    model = mb.RegressionModel.from_bytes(data)
    assert model.to_bytes() == data
    assert model.schema is not None and len(model.trees) >= 1


def test_save_load(tmp_path):
    data = _golden_files()[2]
    model = mb.RegressionModel.from_bytes(data)
    path = tmp_path / "model.mpsb"
    model.save(str(path))
    assert path.read_bytes() == data
    assert sorted(os.listdir(tmp_path)) == ["model.mpsb"]  # no temporary file left behind
    loaded = mb.RegressionModel.load(str(path))
    assert loaded.to_bytes() == data
    with pytest.raises(mb.TrainingError, match="open"):
        mb.RegressionModel.load(str(tmp_path / "absent.mpsb"))
    with pytest.raises(mb.TrainingError):
        model.save(str(tmp_path / "no_such_dir" / "m.mpsb"))


def _payload_offsets(data: bytes):
    """Byte offsets of the first tree's first node inside the payload."""
    p = data[32:]
    features = struct.unpack_from("<I", p, 0)[0]
    nb = struct.unpack_from("<Q", p, 44)[0]
    off = 52 + features * 24 + nb * 4  # tree count
    return p, off + 4 + 4  # first node (after tree count and node count)


def _corrupt(data: bytes):
    p, node = _payload_offsets(data)
    yield "integrity", data[:40] + bytes([data[40] ^ 1]) + data[41:]
    yield "magic", b"X" + data[1:]
    yield "truncated", data[:20]
    yield "major", data[:8] + struct.pack("<H", 2) + data[10:]
    yield "incompatible", data[:12] + struct.pack("<I", 1) + data[16:]
    yield "length", data[:16] + struct.pack("<Q", len(p) + 1) + data[24:]
    yield "trailing", _refresh(data, p + b"\0")
    yield "truncated", _refresh(data, p[:-3])
    bad = bytearray(p)
    bad[node + 34] = 1  # a reserved byte of the first node
    yield "reserved", _refresh(data, bytes(bad))
    bad = bytearray(p)
    bad[node + 32] = 2  # default_left
    yield "default_left", _refresh(data, bytes(bad))
    bad = bytearray(p)
    struct.pack_into("<d", bad, 8, float("nan"))  # base score
    yield "finite", _refresh(data, bytes(bad))
    bad = bytearray(p)
    struct.pack_into("<I", bad, node + 4, 4000)  # root threshold beyond its feature's bins
    yield "threshold", _refresh(data, bytes(bad))
    bad = bytearray(p)
    struct.pack_into("<I", bad, node + 8, 0)  # root's left child = root: a cycle
    yield "cycle", _refresh(data, bytes(bad))
    bad = bytearray(p)
    struct.pack_into("<I", bad, 24, 9)  # objective code
    yield "objective", _refresh(data, bytes(bad))


@pytest.mark.parametrize("kind", [k for k, _ in _corrupt(_golden_files()[0])])
def test_rejects_malformed_files(kind, request):
    data = _golden_files()[0]
    variants = [v for k, v in _corrupt(data) if k == kind]
    for v in variants:
        with pytest.raises(mb.TrainingError, match=kind if kind not in ("length", "magic", "major", "incompatible",
                                                                        "cycle") else None):
            mb.RegressionModel.from_bytes(v)
        try:
            ref = request.getfixturevalue("reference")
        except pytest.skip.Exception:
            continue
        import oracle

        with pytest.raises(oracle.OracleError):
            ref.model_from_bytes(v)


def test_rejects_bad_schema():
    data = _golden_files()[2]
    p = bytearray(data[32:])
    features = struct.unpack_from("<I", p, 0)[0]
    first = 52 + features * 24  # first boundary; make the second equal to it
    count0 = struct.unpack_from("<I", p, 52 + 8)[0]
    assert count0 >= 2
    p[first + 4:first + 8] = p[first:first + 4]
    with pytest.raises(mb.DataError, match="increasing"):
        mb.RegressionModel.from_bytes(_refresh(data, bytes(p)))


def _downgrade(data: bytes, minor: int) -> bytes:
    """Re-encode a 1.4 file in the layout of an older minor version."""
    p = data[32:]
    features, max_bins = struct.unpack_from("<II", p, 0)
    out = bytearray(p[:24])  # features, max_bins, base, learning rate
    pos = 24
    objective = p[pos:pos + 4]
    pos += 4
    alpha_power = p[pos:pos + 16]
    pos += 16
    if minor >= 1:
        out += objective
    if minor >= 4:
        out += alpha_power
    nb = struct.unpack_from("<Q", p, pos)[0]
    out += p[pos:pos + 8]
    pos += 8
    for _ in range(features):
        out += p[pos:pos + 16]
        if minor >= 2:
            out += p[pos + 16:pos + 24]
        pos += 24
    out += p[pos:pos + 4 * nb]
    pos += 4 * nb
    n_trees = struct.unpack_from("<I", p, pos)[0]
    out += p[pos:pos + 4]
    pos += 4
    for _ in range(n_trees):
        n_nodes = struct.unpack_from("<I", p, pos)[0]
        out += p[pos:pos + 4]
        pos += 4
        for _ in range(n_nodes):
            node = p[pos:pos + 40]
            pos += 40
            out += node[:32]
            if minor >= 2:
                out += node[32:40]
            else:
                out += node[33:34] + bytes(7)  # flags, 7 reserved
    head = data[:8] + struct.pack("<HH", 1, minor) + data[12:16]
    return _refresh(head + bytes(16), bytes(out))


@pytest.mark.parametrize("minor", [1, 3])
def test_reads_older_minor_versions(minor, request):
    data = _golden_files()[1]  # squared error, missing values
    old = _downgrade(data, minor)
    model = mb.RegressionModel.from_bytes(old)
    new = mb.RegressionModel.from_bytes(data)
    assert model.base_score == new.base_score
    for t1, t2 in zip(model.trees, new.trees):
        assert np.array_equal(t1["feature_index"], t2["feature_index"])
        assert np.array_equal(t1["leaf_value"], t2["leaf_value"])
    if minor < 2:
        assert not model.schema["missing_counts"].any()
        assert (np.concatenate(model.trees)["default_left"] == 1).all()
    assert model.objective_alpha == 0.5 and model.tweedie_variance_power == 1.5
    try:
        ref = request.getfixturevalue("reference")
    except pytest.skip.Exception:
        return
    theirs = ref.model_from_bytes(old)
    for t1, t2 in zip(theirs.trees, model.trees):
        assert t1.tobytes() == np.ascontiguousarray(t2).tobytes()


def test_softmax_bytes_equal_reference(reference):
    rng = np.random.default_rng(77)
    x = rng.normal(size=(400, 4)).astype(np.float32)
    x[rng.random(x.shape) < 0.05] = np.nan
    y = (np.nan_to_num(x) @ rng.normal(size=(4, 3)) + rng.gumbel(size=(400, 3))).argmax(1).astype(np.float64)
    ds = reference.quantize_dense(x, 16)
    model = reference.train_softmax(ds, y, 3, n_estimators=2, learning_rate=0.4, max_depth=3)
    want = reference.softmax_to_bytes(model)
    ours = mb.MulticlassModel(model.base_scores, 0.4, model.trees)
    assert ours.to_bytes(ds) == want
    back = mb.MulticlassModel.from_bytes(want)
    assert back.base_scores.tobytes() == model.base_scores.tobytes()
    assert np.array_equal(back.class_labels, [0.0, 1.0, 2.0])
    for t1, t2 in zip(back.trees, model.trees):
        assert t1.tobytes() == t2.tobytes()
    theirs = reference.softmax_from_bytes(ours.to_bytes(ds))
    for t1, t2 in zip(theirs.trees, model.trees):
        assert t1.tobytes() == t2.tobytes()
    with pytest.raises(mb.TrainingError, match="multiclass"):
        mb.MulticlassModel.from_bytes(_golden_files()[0])
