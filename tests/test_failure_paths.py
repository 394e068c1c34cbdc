"""Failure detection without a GPU fault.

Every wait of the tile pipeline (consumers on a staged tile, the producer on a
free stage) is bounded; a wait that runs out sets the device error flag and
the kernel returns with nothing in flight, and the host turns the flag into
SFWI_E_CUDA.  sfwi_wait_selftest runs the real pipeline with a producer that
stages nothing and a short bound, so those waits run out; the handle must
report it like a failed run and then keep producing the same results.
"""
import numpy as np
import pytest

from tests.golden.make_golden import load_case
from tests.helpers import make_engine, run_ref_api

pytestmark = pytest.mark.gpu
KEYS = ("syn_z", "syn_x", "res_z", "res_x", "grad_pp", "grad_ps", "illum")


@pytest.mark.parametrize("shape", ["16x32", "8x32c2s3"])
def test_pipeline_wait_timeout_is_reported_and_the_handle_stays_usable(shape):
    import sfwi_gb300 as sg
    shot, inputs, _ = load_case("s1_full")
    fd = make_engine(shot, inputs)
    fd.set_tile_shape(shape)
    first = run_ref_api(shot, inputs, fd=fd)
    with pytest.raises(sg.SfwiError, match="wait timed out"):
        fd.wait_selftest(4096)
    # the context and the handle still work, and give the same results
    fd.imagebuffer_resettozero()
    again = run_ref_api(shot, inputs, fd=fd)
    fd.close()
    for k in KEYS:
        assert np.array_equal(again[k], first[k]), k


def test_wait_selftest_needs_a_batch_and_a_sane_bound():
    import sfwi_gb300 as sg
    shot, inputs, _ = load_case("s1_window")
    fd = make_engine(shot, inputs)
    with pytest.raises(sg.SfwiError, match="run a batch"):
        fd.wait_selftest(4096)
    run_ref_api(shot, inputs, fd=fd)
    with pytest.raises(sg.SfwiError, match="tries"):
        fd.wait_selftest(0)
    fd.close()


def test_plain_runs_refuse_shots_of_other_lengths():
    """records queued for run_models with another length are not read as
    [ntr, nt] by a plain run: the run is refused and the queue dropped"""
    import sfwi_gb300 as sg
    shot, inputs, _ = load_case("s1_full")
    fd = make_engine(shot, inputs)
    nt = shot["nt"]
    gc = np.asarray(inputs["gc"], np.int32)
    fd.enqueue_shot(shot["nx"], shot["isx"], shot["isz"], shot["igz"], shot["ngx_left"], shot["delta_left"], 0, gc,
                    nt=nt - 5)
    with pytest.raises(sg.SfwiError, match="run_models"):
        fd.run()
    with pytest.raises(sg.SfwiError, match="no shots queued"):
        fd.run()
    fd.close()

