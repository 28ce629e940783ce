"""The non-allocating smoother entry point against the hierarchy's own smoother.

olgpu_smooth_box_noalloc serves callers that cannot allocate device memory
(codes that own all device memory through their own pool, or that fix their
memory budget at start-up): they pass one box's fields and the library keeps
the kernel's scratch in a fixed device array.  Here a box is taken from a
hierarchy after one V-cycle, its fields are copied into caller-owned device
memory, and two calls in a row must give the same u as the hierarchy's
smoother (olgpu_time_smoother) run on the same box from the same state.

This file is collected last, so a run that stops at the first failure has run
every other test before it.
"""
import numpy as np
import pytest

from tests.cases import problem

U_TOL = 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["o2_single", "o4_spin", "o8_offset", "sf_binary"])
def test_noalloc_smoother_matches_hierarchy(case):
    torch = pytest.importorskip("torch")
    import ollipticid_gb300 as og

    P = problem(case)
    with og.Elliptic(P) as E:
        E.FASN()
        level = E.mgrid_levels                      # the base grid: one box
        assert E.Get_num_dom(level) == 1
        g = E.box_index(level, 0)
        box = E.boxes[g]
        names = ["u", "b", "c", "rho"] + (["d", "e"] if P.equation != "Punctures" else [])
        dev = {k: torch.from_numpy(E.get_field(g, k)).to("cuda") for k in names}
        torch.cuda.synchronize()
        for call in range(2):
            E.time_smoother(level, 3)               # existing entry point, on the hierarchy
            norms = og.smooth_box_noalloc(dev["u"].data_ptr(), dev["b"].data_ptr(), dev["c"].data_ptr(),
                                          dev["rho"].data_ptr(), box.n, box.order, box.d, 3,
                                          dev["d"].data_ptr() if "d" in dev else 0,
                                          dev["e"].data_ptr() if "e" in dev else 0)
            torch.cuda.synchronize()
            want = E.get_field(g, "u")
            got = dev["u"].cpu().numpy()
            err = float(np.max(np.abs(got - want)))
            assert err <= U_TOL, f"call {call}: max|du| = {err:.3e}"
            assert len(norms) == 3 and all(np.isfinite(norms)) and all(x > 0 for x in norms)


@pytest.mark.gpu
def test_noalloc_rejects_too_many_sweeps():
    torch = pytest.importorskip("torch")
    import ollipticid_gb300 as og
    from ollipticid_gb300 import _abi

    t = torch.zeros(9 * 9 * 9, dtype=torch.float64, device="cuda")
    with pytest.raises(og.OlgpuError) as exc:
        og.smooth_box_noalloc(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), (9, 9, 9), 2,
                              (1.0, 1.0, 1.0), _abi.NOALLOC_MAX_SWEEPS + 1)
    assert exc.value.status == _abi.ERR_INVALID_ARG
    assert "sweeps" in str(exc.value)
