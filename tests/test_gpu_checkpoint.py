"""Checkpoint / resume on the GPU: a run interrupted at t = 1.0 s, written to a checkpoint file, read
back into a new device context (``epgpu_upload`` of the loaded arrays is the resume) and continued to
1.6 s ends in the state of the uninterrupted device run, bit for bit.

Covered: the FP64 step and the deterministic mixed step (no floating-point atomics, so two runs of it
are bitwise identical), each with the std, TPIC (which carries the previous step's ∇v) and APIC
(Bᵢⱼ and Dᵢⱼ) transfers.  The resume path resets the device control block, rebuilds the mixed step's
cell lists from the FP64 positions (``mixed_import``) and the friction-angle cache.
"""
import copy

import numpy as np
import pytest

from conftest import POINT_FIELDS

pytestmark = pytest.mark.gpu

C1 = ([64.1584, 16.0396], [40, 10])
FIELDS = POINT_FIELDS + ["epV", "c0", "phi", "Omega0", "rho0"]


def _instr(cfg, precision):
    instr = copy.deepcopy(cfg["instr"])
    if precision != "fp64":
        instr["gpu"] = {"precision": precision, "jaumann": False, "deterministic": True}
    return instr


@pytest.mark.parametrize("precision", ["fp64", "mixed_df"])
@pytest.mark.parametrize("trsfr", ["std", "tpic", "apic"])
def test_gpu_resume_continues_bit_for_bit(tmp_path, precision, trsfr):
    from epgpu import Engine, checkpoint, ic_slump
    fw = {"deform": "finite", "trsfr": trsfr, "C_pf": 0.99, "musl": True, "locking": True, "damping": 0.1}
    ic, cfg = ic_slump(*C1, fwrk=fw, nonloc={"status": precision == "fp64", "ls": 0.5})
    instr = _instr(cfg, precision)
    # uninterrupted: 1.0 s elastic, then plastic to 1.6 s; the state at 1.0 s is the checkpoint
    e = Engine(copy.deepcopy(ic), instr)
    t, _ = e.run(0, 1.0, 10.0, 0.0)
    mid = e.download()
    t, _ = e.run(1, 1.6, 10.0, t)
    ref = e.download()
    e.close()
    assert (ref.dlam != 0).sum() > 0
    # interrupted at 1.0 s: written, read back into a new context, continued
    time = dict(ic["time"])
    time["t"] = np.array([1.0, ic["time"]["t"][1]])
    m, time2 = checkpoint.load(checkpoint.save(str(tmp_path / "mid.npz"), mid, time))
    e2 = Engine({**ic, "mpts": m}, instr)
    t2, _ = e2.run(1, 1.6, 10.0, float(time2["t"][0]))
    got = e2.download()
    e2.close()
    assert t2 == t
    fields = FIELDS + (["Bij", "Dij"] if trsfr == "apic" else [])
    if precision != "fp64":
        fields = [f for f in fields if f != "Dij"]      # the mixed step does not form Dᵢⱼ
    bad = [f for f in fields if not np.array_equal(np.asarray(getattr(got, f)), np.asarray(getattr(ref, f)))]
    assert not bad, bad


def test_apic_upload_without_affine_state_is_refused():
    """With APIC the step reads Bᵢⱼ and Dᵢⱼ: an upload without them fails instead of keeping stale
    values on the device."""
    from epgpu import Engine, ic_slump
    from epgpu.abi import EPError
    fw = {"deform": "finite", "trsfr": "apic", "C_pf": 0.99, "musl": True, "locking": True, "damping": 0.1}
    ic, cfg = ic_slump(*C1, fwrk=fw)
    e = Engine(copy.deepcopy(ic), cfg["instr"])
    m = ic["mpts"].copy()
    m.Bij = None
    with pytest.raises(EPError) as ex:
        e.upload(m)
    assert ex.value.status == 1 and "Bij" in str(ex.value)
    e.close()
