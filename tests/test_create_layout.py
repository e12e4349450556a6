"""Output layout of a PAR2 create (ParPar's defaults, lib/par2gen.js) — host
logic only: volume sizes and names, critical packet repetition, display names."""
import math

from parpar_gb300.create import display_names, js_round, plan_files, pow2_volumes, volume_name


def _kinds(of):
    return "".join({"recovery": "R", "crit": "c", "creator": "C"}[k] for k, _ in of.packets)


def test_js_round_halves_up():
    assert [js_round(x) for x in (0.5, 1.5, 2.5, 2.4999, 0.0)] == [1, 2, 3, 2, 0]


def test_pow2_volumes_and_names():
    assert pow2_volumes(10) == [(1, 0), (2, 1), (4, 3), (3, 7)]
    assert pow2_volumes(1) == [(1, 0)]
    assert pow2_volumes(0) == []
    assert pow2_volumes(20, max_slices=4) == [(1, 0), (2, 1), (4, 3), (4, 7), (4, 11), (4, 15), (1, 19)]
    assert volume_name(3, 7, 10) == ".vol07+03.par2"
    assert volume_name(1, 0, 5) == ".vol00+01.par2"
    assert volume_name(512, 511, 1023) == ".vol0511+0512.par2"
    assert volume_name(0, 0, 10) == ".par2"


def test_plan_repeats_critical_packets_log2():
    files = plan_files("x", 3, 10)
    assert [f.name for f in files] == ["x.par2", "x.vol00+01.par2", "x.vol01+02.par2", "x.vol03+04.par2",
                                       "x.vol07+03.par2"]
    assert [_kinds(f) for f in files] == ["cccC", "RcccC", "RccRcC", "RccRcRccRcC", "RccRccRccC"]
    # every volume: its recovery exponents in order, copies = max(round(log2 n), 1)
    for f in files[1:]:
        exps = [k for kind, k in f.packets if kind == "recovery"]
        assert exps == list(range(exps[0], exps[0] + len(exps)))
        copies = max(js_round(math.log(len(exps)) / math.log(2)), 1)
        assert sum(1 for kind, _ in f.packets if kind == "crit") == 3 * copies
        assert f.packets[-1] == ("creator", None)


def test_plan_single_file_and_no_index():
    only = plan_files("y", 2, 0)
    assert [f.name for f in only] == ["y.par2"] and _kinds(only[0]) == "ccC"
    vol = plan_files("z", 2, 1, index=False)
    assert [f.name for f in vol] == ["z.par2"] and _kinds(vol[0]) == "RccC"


def test_display_names_common_root(tmp_path):
    a = tmp_path / "d1" / "a.bin"
    b = tmp_path / "d1" / "sub" / "b.bin"
    assert display_names([str(a), str(b)]) == ["a.bin", "sub/b.bin"]
    assert display_names([str(a)]) == ["a.bin"]
    assert display_names(["/x/p", "/y/q"]) == ["x/p", "y/q"]
