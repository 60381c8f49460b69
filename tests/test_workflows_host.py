"""Host-side parts of the list workflows (rascil_gb300/workflows.py): the
rsexecute stand-in, zero / subtract / sum_predict / remove_sumwt semantics
(rascil/workflows/rsexecute/imaging/imaging_rsexecute.py:844-910,
rascil/processing_components/imaging/imaging_helpers.py:45-72), and the
block map's order and error behaviour.  No GPU."""
import numpy
import pytest


def _blocks(n=3):
    from rascil_gb300 import simulation as sim
    uvw, f, pc, cfg = sim.observation("small-array", ntimes=2)
    out = []
    for i in range(n):
        b = sim.make_blockvisibility(uvw, f, pc, cfg)
        b["vis"].data[...] = i + 1.0
        out.append(b)
    return out


def test_rsexecute_stand_in_runs_immediately():
    from rascil_gb300.workflows import rsexecute
    f = rsexecute.execute(lambda x, y=1: x + y, nout=1)
    assert rsexecute.compute([f(1), f(2, y=5)], sync=True) == [2, 7]
    assert rsexecute.persist("g") == "g" and rsexecute.optimize([1]) == [1]
    rsexecute.set_client(use_dask=False)
    rsexecute.close()


def test_zero_list_copy_and_in_place():
    from rascil_gb300.workflows import zero_list_rsexecute_workflow
    blocks = _blocks()
    z = zero_list_rsexecute_workflow(blocks)
    assert all(numpy.all(b["vis"].data == 0) for b in z)
    assert all(numpy.all(b["vis"].data == i + 1) for i, b in enumerate(blocks))
    z = zero_list_rsexecute_workflow(blocks + [None], copy=False)
    assert z[:3] == blocks and z[3] is None
    assert all(numpy.all(b["vis"].data == 0) for b in blocks)


def test_subtract_and_sum_predict_results():
    from rascil_gb300.workflows import (remove_sumwt, subtract_list_rsexecute_workflow,
                                        sum_predict_results, sum_predict_results_rsexecute)
    blocks = _blocks()
    d = subtract_list_rsexecute_workflow(blocks, blocks[::-1])
    numpy.testing.assert_array_equal(d[0]["vis"].data, -2.0)
    numpy.testing.assert_array_equal(blocks[0]["vis"].data, 1.0)
    assert subtract_list_rsexecute_workflow([None], [blocks[0]]) == [None]
    s = sum_predict_results([None] + blocks)
    assert s is blocks[0]
    numpy.testing.assert_array_equal(s["vis"].data, 6.0)
    t = sum_predict_results_rsexecute(_blocks())
    numpy.testing.assert_array_equal(t["vis"].data, 6.0)
    assert remove_sumwt([("a", 1), ("b", 2)]) == ["a", "b"]


def test_block_map_keeps_order_and_raises():
    from rascil_gb300.workflows import _map_blocks
    assert _map_blocks(lambda x: x * x, range(7), 4) == [x * x for x in range(7)]

    def bad(x):
        if x == 3:
            raise ValueError("block 3")
        return x

    with pytest.raises(ValueError, match="block 3"):
        _map_blocks(bad, range(6), 3)
