"""Host-side ownership in the Python binding: a context closes the bodies and servers made on it
before it is destroyed, so no body is freed after its context (b3g_body_destroy reads its
context). Runs on CPU against a fake library that records the calls."""
import ctypes as C

from bounce_softbody_gb300 import b3g, meshes


class FakeLib:
    def __init__(self):
        self.calls = []
        self.next = 100

    def _new(self, out):
        self.next += 1
        C.cast(out, C.POINTER(C.c_void_p))[0] = self.next
        return 0

    def b3g_context_create(self, device, out):
        self.calls.append("context_create")
        return self._new(out)

    def b3g_body_create(self, ctx, desc, out):
        self.calls.append("body_create")
        return self._new(out)

    def b3g_server_create(self, ctx, budget, max_active, dt, cfg, out):
        self.calls.append("server_create")
        return self._new(out)

    def b3g_solver_config_default(self, cfg):
        return None

    def b3g_context_destroy(self, h):
        self.calls.append("context_destroy")
        return 0

    def b3g_body_destroy(self, h):
        self.calls.append("body_destroy")
        return 0

    def b3g_server_destroy(self, h):
        self.calls.append("server_destroy")
        return 0


def test_context_close_destroys_dependents_first(monkeypatch):
    fake = FakeLib()
    monkeypatch.setattr(b3g, "load_library", lambda *a, **k: fake)
    ctx = b3g.Context(0)
    desc = meshes.tet_grid(2, 2, 2)
    bodies = [b3g.Body(ctx, desc) for _ in range(2)]
    srv = b3g.Server(ctx, 1 << 20, 4, 1 / 60)
    ctx.close()
    assert fake.calls[-1] == "context_destroy"
    assert fake.calls.index("server_destroy") < fake.calls.index("body_destroy")
    assert fake.calls.count("body_destroy") == 2
    # closing again later (or at garbage collection) does not reach the library
    n = len(fake.calls)
    for b in bodies:
        b.close()
    srv.close()
    ctx.close()
    assert len(fake.calls) == n
