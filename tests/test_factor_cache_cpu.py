"""Host logic of engine.Factor's handle reuse on the CPU, with the C ABI
replaced by a fake that hands out integer handles: a released factor of a
process-wide symbolic is parked and taken by the next factor of the same
key, at most one is parked per key (others are destroyed), and a creation
that reports FDFD_ERR_OOM frees the parked factors and is retried once."""
import ctypes as C

import pytest
import torch

from fdfdpy_gb300 import engine
from fdfdpy_gb300 import _native as N


class _FakeABI:
    def __init__(self):
        self.next, self.created, self.destroyed, self.oom = 1, [], [], 0

    def call(self, name, *args):
        if name == "fdfd_factor_create":
            if self.oom:
                self.oom -= 1
                raise N.FDFDError(N.FDFD_ERR_OOM, "factor_create: device allocation failed")
            args[-1]._obj.value = self.next
            self.created.append(self.next)
            self.next += 1

    def lib(self):
        abi = self

        class L:
            @staticmethod
            def fdfd_factor_destroy(h):
                abi.destroyed.append(h.value if isinstance(h, C.c_void_p) else h)
        return L


class _Sym:
    Nx, Ny, leaf_area, batch, handle = 6, 5, 64, 1, None


@pytest.fixture
def abi(monkeypatch):
    fake = _FakeABI()
    monkeypatch.setattr(engine.N, "call", fake.call)
    monkeypatch.setattr(engine.N, "lib", fake.lib)
    monkeypatch.setattr(engine, "device", lambda: torch.device("cpu"))

    class _Cur:
        cuda_stream = 0

        def wait_event(self, ev):
            pass
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a: _Cur())
    emptied = []
    monkeypatch.setattr(torch.cuda, "empty_cache", lambda: emptied.append(1))
    fake.emptied = emptied
    sym = _Sym()
    monkeypatch.setitem(engine._sym_cache, (6, 5, 64), sym)
    monkeypatch.setattr(engine, "_parked", {})
    yield fake, sym
    engine._parked.clear()


def _h(f):
    return f.handle.value


def test_released_factor_is_reused_and_one_is_kept_per_key(abi):
    fake, sym = abi
    f1 = engine.Factor(sym, "c64")
    assert fake.created == [1]
    del f1                                   # parked
    f2 = engine.Factor(sym, "c64")           # takes handle 1
    f3 = engine.Factor(sym, "c64")           # nothing parked: a new one
    assert (_h(f2), _h(f3)) == (1, 2) and fake.created == [1, 2]
    g = engine.Factor(sym, "c128")           # another key: its own handle
    assert _h(g) == 3
    del f2, f3                               # 1 parked, 2 destroyed (one per key)
    assert fake.destroyed == [2]
    engine.release_cached_factors()
    assert fake.destroyed == [2, 1] and not engine._parked


def test_out_of_memory_frees_parked_factors_and_retries_once(abi):
    fake, sym = abi
    other = engine.Factor(sym, "c128")
    del other                                # parked under the complex128 key
    fake.oom = 1
    f = engine.Factor(sym, "c64")            # OOM, parked ones freed, retried
    assert fake.destroyed == [1] and fake.emptied == [1] and _h(f) == 2
    fake.oom = 2
    with pytest.raises(N.FDFDError) as e:
        engine.Factor(sym, "c64")            # fails again after the retry: reported
    assert e.value.code == N.FDFD_ERR_OOM
