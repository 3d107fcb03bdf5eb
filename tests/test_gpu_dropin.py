"""The reference-named drop-in symbols (include/cmc_dropin.h) driven in the
reference's main-loop order (cmc.c:152-167, 240-407) on a host star[] array
of records, against the same kernels through the cmcg_* API: identical bits
in every host field the replaced functions write, and whole records carried
through the sort."""
import ctypes as C

import numpy as np
import pytest

import cmcgpu

pytestmark = pytest.mark.gpu

# a star_t-like record: the hot fields at the offsets numpy chooses, plus
# fields the device never sees (they must travel with their star in the sort)
STAR = np.dtype([("r", "f8"), ("vr", "f8"), ("vt", "f8"), ("m", "f8"), ("E", "f8"), ("J", "f8"), ("id", "i8"),
                 ("rnew", "f8"), ("vrnew", "f8"), ("vtnew", "f8"), ("rOld", "f8"), ("X", "f8"), ("Y", "f8"),
                 ("r_peri", "f8"), ("r_apo", "f8"), ("se_k", "i4"), ("payload", "f8", (5,))], align=True)
SCALARS = ("Dt", "Mtotal", "Rtidal", "max_r", "Eescaped", "Jescaped", "TidalMassLoss", "Etidal", "Etot", "KE", "PE")


class Host:
    """The reference's globals for one cluster, in numpy memory."""

    def __init__(self, ic, N, sync_each=1):
        dim = N + 2
        self.star = np.zeros(dim, STAR)
        s = self.star
        s["r"][1:N + 1] = ic["r"]
        s["m"][1:N + 1] = ic["m"] * float(N)  # stored x N_STAR (cmc_fits.c:99)
        s["vr"][1:N + 1] = ic["vr"]
        s["vt"][1:N + 1] = ic["vt"]
        s["id"][1:N + 1] = ic["id"]
        s["se_k"][1:N + 1] = (ic["id"] % 15).astype(np.int32)
        s["payload"][1:N + 1] = ic["id"][:, None] * np.arange(1, 6)[None, :] + 0.5
        self.star_r = np.zeros(dim)
        self.star_m = np.zeros(dim)
        self.star_phi = np.zeros(dim)
        self.star_r[1:N + 1] = s["r"][1:N + 1]
        self.star_m[1:N + 1] = s["m"][1:N + 1]
        self.star_r[0], self.star_r[N + 1] = 1e-20, 1e10
        self.N_MAX = np.array([N], np.int64)
        self.N_MAX_NEW = np.array([N], np.int64)
        self.tcount = np.array([1], np.int64)
        self.sc = {k: np.zeros(1) for k in SCALARS}
        h = cmcgpu.DropinHost()
        L = cmcgpu.dropin_lib()
        L.cmcx_default_host(C.byref(h))
        h.star, h.star_size = s.ctypes.data, STAR.itemsize
        for f in ("r", "vr", "vt", "m", "E", "J", "id", "rnew", "vrnew", "vtnew", "rOld", "X", "Y", "r_peri",
                  "r_apo"):
            setattr(h, f"off_{f}", STAR.fields[f][1])
        h.id_bytes = 8
        h.star_r, h.star_m, h.star_phi = (a.ctypes.data for a in (self.star_r, self.star_m, self.star_phi))
        h.N_STAR_DIM = dim
        h.N_MAX, h.N_MAX_NEW, h.tcount = self.N_MAX.ctypes.data, self.N_MAX_NEW.ctypes.data, self.tcount.ctypes.data
        for k in SCALARS:
            setattr(h, k, self.sc[k].ctypes.data)
        h.sync_each = sync_each
        self.h = h

    def field(self, name):
        return self.star[name][1:int(self.N_MAX_NEW[0]) + 1].copy()


@pytest.fixture
def dropin(gpulib):
    L = gpulib.dropin_lib()
    errors = []
    handler = gpulib.ABORT_HANDLER(lambda code, where: errors.append((code, where.decode())))
    L.cmcx_set_abort(handler)
    yield L, errors
    L.cmcx_unbind()
    L.cmcx_set_abort(gpulib.ABORT_HANDLER())


def _setup(gpulib, model, N, imf, sync_each=1):
    ic = gpulib.generate(model, N, seed=N + 3, imf=imf)
    p = gpulib.default_params(N_STAR=N, orbit_r=ic["rtid"], seed=99)
    host = Host(ic, N, sync_each)
    ref = gpulib.Context([N], p)
    ref.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    return ic, p, host, ref


@pytest.mark.parametrize("model,N,imf", [(cmcgpu.KING, 6000, 1), (cmcgpu.PLUMMER, 5001, 0)])
def test_dropin_main_loop_matches_the_c_abi(gpulib, dropin, model, N, imf):
    L, errors = dropin
    ic, p, host, ref = _setup(gpulib, model, N, imf)
    assert L.cmcx_bind(C.byref(host.h), C.byref(p)) == 0
    # start-up, cmc.c:152-167
    L.calc_potential_new()
    L.compute_energy_new()
    ref.initialize()
    assert np.array_equal(host.star_phi[:N + 2], ref.get("star_phi"))
    assert np.array_equal(host.field("E"), ref.get("E")) and np.array_equal(host.field("J"), ref.get("J"))
    for step in range(3):
        host.tcount[0] = step + 1
        if step:
            ref.end_step()
        # main loop body, cmc.c:258-350
        L.calc_timestep(None)
        ref.begin_step()
        ref.calc_timestep()
        assert host.sc["Dt"][0] == ref.scalar("Dt")
        L.dynamics_apply(host.sc["Dt"][0], None)
        ref.dynamics_apply(ref.scalar("Dt"))
        for hf, rf in (("vr", "vr_rel"), ("vt", "vt_rel"), ("E", "E"), ("J", "J"), ("Y", "Y")):
            assert np.array_equal(host.field(hf), ref.get(rf)), (step, hf)
        L.energy_conservation1()
        L.new_orbits_calculate()
        L.energy_conservation2()
        ref.new_orbits_calculate()
        for f in ("rnew", "vrnew", "vtnew", "X", "r_peri", "r_apo"):
            assert np.array_equal(host.field(f), ref.get(f)), (step, f)
        assert host.sc["max_r"][0] == ref.scalar("max_r")
        L.tidally_strip_stars()
        ref.tidally_strip_stars()
        assert np.array_equal(host.field("rnew"), ref.get("rnew"))
        assert host.sc["Rtidal"][0] == ref.scalar("Rtidal")
        before = {int(i): (int(k), tuple(pl)) for i, k, pl in
                  zip(host.field("id"), host.field("se_k"), host.field("payload"))}
        L.ComputeIntermediateEnergy()
        L.qsorts_new()
        L.post_sort_comm()
        ref.qsorts_new()
        n = ref.nstars()
        assert host.N_MAX_NEW[0] == n and host.N_MAX[0] == n
        assert np.array_equal(host.field("id"), ref.ids())
        for i, k, pl in zip(host.field("id"), host.field("se_k"), host.field("payload")):
            assert before[int(i)] == (int(k), tuple(pl))  # the whole record moved
        for f in ("r", "m", "vr", "vt", "rOld"):
            assert np.array_equal(host.field(f), ref.get(f)), (step, f)
        assert np.array_equal(host.star_r[:n + 2], ref.get("star_r"))
        assert np.array_equal(host.star_m[:n + 2], ref.get("star_m"))
        assert L.potential_calculate() == n
        ref.calc_potential()
        assert np.array_equal(host.star_phi[:n + 2], ref.get("star_phi"))
        assert host.sc["Mtotal"][0] == ref.scalar("Mtotal")
        L.energy_conservation3()
        ref.energy_conservation3()
        assert np.array_equal(host.field("vr"), ref.get("vr")) and np.array_equal(host.field("vt"), ref.get("vt"))
        L.compute_energy_new()
        ref.compute_energy()
        assert np.array_equal(host.field("E"), ref.get("E")) and np.array_equal(host.field("J"), ref.get("J"))
        assert host.sc["Etot"][0] == ref.scalar("Etot")
        for r in (0.0, 0.3, 2.0, 1e3):
            assert L.potential(r) == ref.potential(r)
    assert not errors
    ref.close()


def test_dropin_lazy_sync_and_download(gpulib, dropin):
    """sync_each = 0: the functions leave star[] alone; cmcx_download brings
    the device state back in one call."""
    L, errors = dropin
    N = 4000
    ic, p, host, ref = _setup(gpulib, cmcgpu.KING, N, 1, sync_each=0)
    assert L.cmcx_bind(C.byref(host.h), C.byref(p)) == 0
    L.calc_potential_new()
    L.compute_energy_new()
    assert not host.star_phi.any() and not host.field("E").any()
    L.calc_timestep(None)
    L.dynamics_apply(host.sc["Dt"][0], None)
    L.new_orbits_calculate()
    L.tidally_strip_stars()
    L.qsorts_new()
    L.calc_potential_new()
    L.energy_conservation3()
    L.compute_energy_new()
    assert L.cmcx_download() == 0
    ref.initialize()
    ref.step(1)
    n = ref.nstars()
    assert host.N_MAX_NEW[0] == n
    assert np.array_equal(host.field("id"), ref.ids())
    for f in ("r", "m", "vr", "vt", "E", "J"):
        assert np.array_equal(host.field(f), ref.get(f)), f
    assert np.array_equal(host.star_phi[:n + 2], ref.get("star_phi"))
    assert not errors
    ref.close()


def test_dropin_device_error_reaches_the_abort_handler(gpulib, dropin):
    """A NaN mass in star[] stops potential_calculate with the reference's
    error code (cmc_utils.c:688), through the handler that replaces exit_cleanly."""
    L, errors = dropin
    N = 4000
    ic, p, host, ref = _setup(gpulib, cmcgpu.PLUMMER, N, 0)
    host.star["m"][77] = np.nan
    host.star_m[77] = np.nan
    assert L.cmcx_bind(C.byref(host.h), C.byref(p)) == 0
    L.calc_potential_new()
    assert errors == [(cmcgpu.CMCG_ERR_NAN_MASS, "potential_calculate")]
    ref.close()
