"""The batched benchmark's generated simulations (no GPU): deterministic per index, within the specified ranges,
and valid inputs for the reference-compatible front end."""
import json
import math

import numpy as np

from umcx_gb300.workloads import EDGES, config5


def test_configs_are_deterministic_and_distinct():
    a = [json.dumps(config5(i)) for i in range(16)]
    b = [json.dumps(config5(i)) for i in range(16)]
    assert a == b
    assert len(set(a)) == 16
    seeds = {config5(i)["Session"]["RNGSeed"] for i in range(256)}
    assert len(seeds) == 256 and all(0 < s < 2 ** 31 for s in seeds)


def test_parameters_within_the_specified_ranges():
    photons, edges, labels, sources = [], set(), set(), set()
    for i in range(256):
        c = config5(i)
        edge = c["Domain"]["Dim"][0]
        assert c["Domain"]["Dim"] == [edge] * 3 and edge in EDGES
        edges.add(edge)
        media = c["Domain"]["Media"]
        assert media[0] == {"mua": 0.0, "mus": 0.0, "g": 1.0, "n": 1.0}
        assert 3 <= len(media) <= 6  # background + 2-5 tissue labels
        labels.add(len(media) - 1)
        for m in media[1:]:
            assert 0.001 <= m["mua"] <= 0.05 and 0.5 <= m["mus"] <= 20.0
            assert 0.0 <= m["g"] <= 0.95 and 1.33 <= m["n"] <= 1.45
        f = c["Forward"]
        assert f["T0"] == 0.0 and f["T1"] == 5e-9 and round((f["T1"] - f["T0"]) / f["Dt"]) == 10
        n = c["Session"]["Photons"]
        assert 1e5 <= n <= 1e7
        photons.append(math.log10(n))
        src = c["Optode"]["Source"]
        sources.add(src["Type"])
        pos, d = np.array(src["Pos"]), np.array(src["Dir"])
        axis = int(np.flatnonzero(d)[0])
        assert np.count_nonzero(d) == 1 and abs(d[axis]) == 1.0
        assert (pos[axis] == 0.0 and d[axis] > 0) or (pos[axis] > edge - 0.01 and d[axis] < 0)  # on a face, inwards
        tags = [next(iter(s.values()))["Tag"] if "ZLayers" not in s else s["ZLayers"][0][2] for s in c["Shapes"]]
        assert tags[0] == 1 and sorted(tags[1:]) == list(range(2, len(media)))
    assert edges == set(EDGES) and labels == {2, 3, 4, 5} and sources == {"pencil", "isotropic"}
    # log-uniform budgets: the mean of log10 is near 6 and both decades are populated
    assert abs(np.mean(photons) - 6.0) < 0.15 and min(photons) < 5.2 and max(photons) > 6.8


def test_configs_parse_through_the_front_end():
    from umcx_gb300 import Job

    for i in range(8):
        job = Job.from_json(config5(i, photon_scale=0.01, max_edge=48))
        s = job.sim
        c = config5(i, photon_scale=0.01, max_edge=48)
        assert (s.dim[0], s.dim[3]) == (c["Domain"]["Dim"][0], 10)
        assert s.mediumnum == len(c["Domain"]["Media"]) and s.isreflect == 1
        assert set(np.unique(job.labels & 0x7F)) <= set(range(1, s.mediumnum))


def test_benchmark_configurations_equal_the_pinned_ones():
    """The benchmark's configurations 1-3 (umcx_gb300.workloads) are the ones the oracle is pinned on
    (tests/golden/make_golden.py), apart from the photon count."""
    import json
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden import C1, C2, C3

    from umcx_gb300.workloads import config1, config2, config3

    for mine, pinned, n in ((config1(), C1, 1000000), (config2(), C2, 10000000), (config3(), C3, 100000000)):
        a = json.loads(json.dumps(mine))
        b = json.loads(json.dumps(pinned))
        assert a["Session"].pop("Photons") == n
        b["Session"].pop("Photons")
        assert a == b
