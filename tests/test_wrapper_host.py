"""The Python wrapper's host logic without a GPU: every context call goes to
a stand-in library that accepts it (returns 0), so the argument marshalling,
option handling and result conversion of the methods the tests, the bench
and smoke() use run on the CPU.  The option defaults come from the real
library (lpm_default_solver_opts needs no device)."""

import numpy as np
import pytest

import cases


class _AcceptAll:
    def __init__(self, real):
        self.real = real
        self.calls = []

    def __getattr__(self, name):
        if name == "lpm_default_solver_opts":
            return self.real.lpm_default_solver_opts
        if name == "lpm_last_error":
            return lambda: b""

        def f(*args):
            self.calls.append((name, args))
            return 0
        return f


@pytest.fixture()
def fake(gpu_lib, monkeypatch):
    lib = _AcceptAll(gpu_lib.load())
    monkeypatch.setattr(gpu_lib, "load", lambda *a, **k: lib)
    return gpu_lib, lib


def test_load_step_returns_every_stat(fake):
    G, lib = fake
    s = G.Specimen(0)
    st = s.load_step(cases.sc_bcs(0.001))
    assert set(st) == {f for f, _ in G.StepStats._fields_}
    assert st["amg_builds"] == 0 and st["status"] == 0
    name, args = lib.calls[-1]
    assert name == "lpm_load_step" and args[1] == len(cases.sc_bcs(0.001))
    x, st2 = s.solve_rhs(np.zeros(12))
    assert x.shape == (12,) and set(st2) == set(st)
    assert set(s.solve()) == set(st)


def test_set_solver_defaults_and_preconditioner(fake):
    G, lib = fake
    s = G.Specimen(0)
    o = s.set_solver(preconditioner=G.PRECOND_AMG, amg_spacing=0.5, cg_rtol=1e-9)
    assert o.preconditioner == G.PRECOND_AMG and o.amg_spacing == 0.5 and o.cg_rtol == 1e-9
    d = G.default_opts()
    assert d.preconditioner == G.PRECOND_BJ and d.amg_spacing == 0.0 and d.amg_rebuild == 2.5
    assert d.amg_sweeps == 1
    assert d.precision == G.PREC_FP64 and d.cg_forcing == 0.0
    with pytest.raises(KeyError):
        s.set_solver(no_such_option=1)
