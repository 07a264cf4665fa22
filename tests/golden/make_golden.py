"""Generate the golden fixtures in tests/golden/ by running the reference's own
Python code (spinifel, mounted read-only at /root/reference in the build
container) on seeded inputs.

The reference cannot be installed as-is here: finufft/cufinufft, skopi,
PyNVTX, callmonitor, toml and matplotlib are absent.  This script stubs only
those imports (identity decorators, tomllib for toml, a Shoemake quaternion
sampler and the eval/geom.py rotation formula for skopi, the FP64 ES oracle of
oracle/nufft.py for the un-vendored finufft) and then calls, unmodified:

  * spinifel.sequential.nearest_neighbor.nearest_neighbor (CPU branch:
    sklearn euclidean_distances + argmin)            -> golden_nn.npz
  * spinifel.sequential.orientation_matching.SNM.slicing_and_match
    (numpy/scipy-dgemm branch)                       -> golden_snm.npz
  * spinifel.sequential.orientation_matching.slicing_and_match
    (function path, global std, nearest_neighbor)   -> golden_sam.npz
  * spinifel.sequential.autocorrelation.Merge.solve_ac (scipy cg)
                                                     -> golden_merge.npz
  * spinifel.autocorrelation.forward / adjoint glue  -> golden_ops.npz
  * spinifel.mpi.autocorrelation.MergeMPI.solve_ac, its ranks run as
    threads over an in-process communicator (gather / bcast / Bcast)
                                                     -> golden_sweep.npz
  * spinifel.sequential.phasing.phase (numpy branch) -> golden_phase.npz
  * spinifel.prep clipping / binning / SAXS on seeded frames and geometry
    (numpy 2 dropped numpy.int, which get_saxs reads; it is set to int)
                                                     -> golden_prep.npz
  * eval.fsc.compute_fsc, eval.align.rotate_volume / score_deformations /
    center_volume / align_volumes (numpy branch; skopi's samplers and
    numpy's global generator seeded)               -> golden_eval.npz
    (numpy 2 dropped numpy.infty, which phase() reads; it is set to inf)

Inputs are regenerated from the stored seeds by tests (numpy PCG64 streams are
stable), so only small outputs are committed.  Run where the reference's
sources are checked out:
    python tests/golden/make_golden.py [path-to-spinifel-checkout]
(or set SPINIFEL_REFERENCE).
"""
from __future__ import annotations

import os
import sys
import tempfile
import tomllib
import types

import numpy as np

# the reference project's checkout: first argument, or SPINIFEL_REFERENCE
REF = (sys.argv[1] if len(sys.argv) > 1 else
       os.environ.get("SPINIFEL_REFERENCE", "/root/reference"))
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import nufft as onufft  # noqa: E402
from tests.golden import cases  # noqa: E402


def _stub_modules(quat_seed: int):
    def annotate(*a, **k):
        def deco(f):
            return f
        return deco

    nvtx = types.ModuleType("PyNVTX")
    nvtx.annotate = annotate
    nvtx.RangePushA = lambda *a, **k: None
    nvtx.RangePop = lambda *a, **k: None
    sys.modules["PyNVTX"] = nvtx

    cm = types.ModuleType("callmonitor")
    cm.intercept = lambda f: f
    sys.modules["callmonitor"] = cm

    toml = types.ModuleType("toml")
    toml.load = lambda path: tomllib.load(open(path, "rb"))
    sys.modules["toml"] = toml

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mcm = types.ModuleType("matplotlib.cm")
    mcol = types.ModuleType("matplotlib.colors")
    mcol.LogNorm = mcol.SymLogNorm = object
    mpl.pyplot, mpl.cm, mpl.colors = plt, mcm, mcol
    sys.modules.update({"matplotlib": mpl, "matplotlib.pyplot": plt, "matplotlib.cm": mcm,
                        "matplotlib.colors": mcol})

    from spinifel_gb300 import geom

    skp = types.ModuleType("skopi")
    skp.quaternion2rot3d = lambda q: geom.quaternion2rot3d(np.asarray(q))
    rng = np.random.default_rng(quat_seed)
    skp.get_uniform_quat = lambda n, avoid_symmetric=True: geom.uniform_quaternions(n, rng)
    skp.get_random_quat = lambda n: geom.uniform_quaternions(n, rng)
    sys.modules["skopi"] = skp

    # spinifel.extern: the package __init__ imports cufinufft unconditionally;
    # provide the two functions autocorrelation.py takes from it (finufft
    # call convention: nufft_3d_t2(x, y, z, ugrid, sign, eps, n),
    # nufft_3d_t1(x, y, z, nuvect, sign, eps, nx, ny, nz)).
    ext = types.ModuleType("spinifel.extern")
    ext.__path__ = [os.path.join(REF, "spinifel", "extern")]

    def t2(x, y, z, ugrid, sign, eps, n):
        out = onufft.nufft3d2(x, y, z, ugrid, sign, 1e-12)
        assert out.size == n
        return out

    def t1(x, y, z, nuvect, sign, eps, nx, ny, nz):
        return onufft.nufft3d1(x, y, z, nuvect, (nx, ny, nz), sign, 1e-12)

    ext.nufft_3d_t1, ext.nufft_3d_t2 = t1, t2
    sys.modules["spinifel.extern"] = ext

    # spinifel.sequential/__init__.py only imports the CLI driver (main.py:
    # HDF5 and psana readers, the cufinufft/finufft dispatch); load the
    # package's modules without running it.
    seq = types.ModuleType("spinifel.sequential")
    seq.__path__ = [os.path.join(REF, "spinifel", "sequential")]
    sys.modules["spinifel.sequential"] = seq


def _settings_file(c: dict) -> str:
    det = "[" + ", ".join(str(v) for v in c["det_shape"]) + "]"
    text = f"""
[debug]
verbose = false
show_image = false
use_callmonitor = false
[runtime]
N_images_per_rank = {c.get("n_images", 10)}
use_cuda = false
use_cufinufft = false
use_cupy = false
use_single_prec = false
[algorithm]
N_clipping = 0
N_binning = 0
N_orientations = {c["n_orient"]}
N_batch_size = {c["batch"]}
oversampling = 1
solve_ac_maxiter = {c.get("maxiter", 100)}
{c.get("extra", "")}[detector]
shape = {det}
"""
    fd, path = tempfile.mkstemp(suffix=".toml")
    with os.fdopen(fd, "w") as f:
        f.write(text)
    return path


class OracleNUFFT:
    """Stands in for spinifel.extern.nufft_ext.NUFFT (finufft 2.1 branch,
    nufft_ext.py:420-487) with the FP64 ES oracle at eps 1e-12."""

    def __init__(self, ref_orientations, ppr, pdr, oversampling=1):
        from spinifel_gb300 import geom

        self.ref_orientations = ref_orientations
        self.mult = np.pi / (oversampling * pdr.max())
        H, K, L = geom.hkl(ref_orientations, ppr)
        self.HKL = np.stack([H, K, L]).reshape(3, len(ref_orientations), -1) * self.mult

    def forward(self, ugrid, st, en, support, use_recip_sym, N):
        H_, K_, L_ = (self.HKL[i, st:en].reshape(-1) for i in range(3))
        if support is not None:
            ugrid = ugrid * support
        return onufft.nufft3d2(H_, K_, L_, ugrid, -1, 1e-12)

    def adjoint(self, nuvect, H_, K_, L_, support, use_reciprocal_symmetry, M):
        ugrid = onufft.nufft3d1(H_, K_, L_, np.asarray(nuvect), (M, M, M), -1, 1e-12)
        ugrid = ugrid * support
        if use_reciprocal_symmetry:
            ugrid = ugrid.real
        return ugrid / M ** 3


class _GetArray(np.ndarray):
    def get(self):
        return np.asarray(self)


def main():
    sys.path.insert(0, REF)
    _stub_modules(cases.QUAT_SEED)

    # --- nearest_neighbor (CPU branch) --------------------------------------
    c = cases.NN
    sys.argv = ["spinifel", "--mode=sequential", "--settings=" + _settings_file(
        {"det_shape": (1, 1, c["n_pix"]), "n_orient": c["n_ref"], "batch": c["n_ref"]})]
    import spinifel.sequential.nearest_neighbor as rnn

    model_slices, slices = cases.nn_inputs()
    idx = rnn.nearest_neighbor(model_slices, slices, c["n_ref"])
    np.savez_compressed(os.path.join(HERE, "golden_nn.npz"), index=idx.astype(np.int32))
    print("nn", idx[:10])

    # --- SNM and the function path -------------------------------------------
    s = cases.SNM
    from spinifel import SpinifelSettings
    st = SpinifelSettings()
    # refresh the singleton with this case's settings file
    sys.argv = ["spinifel", "--mode=sequential", "--settings=" + _settings_file(
        {"det_shape": s["det_shape"], "n_orient": s["n_orient"], "batch": s["batch"]})]
    st._SpinifelSettings__toml = sys.argv[2].split("=", 1)[1]
    st._SpinifelSettings__params = []
    st.refresh()
    import spinifel.sequential.orientation_matching as rom

    ac, ppr, pdr, quats, slices_ = cases.snm_inputs()
    nufft = OracleNUFFT(quats, ppr, pdr)
    snm = rom.SNM(st, slices_, ppr, pdr, nufft)
    q_snm = snm.slicing_and_match(ac.copy())
    idx_snm = np.array([np.flatnonzero((quats == q).all(axis=1))[0] for q in q_snm])
    dist = np.array(snm.dist)
    np.savez_compressed(os.path.join(HERE, "golden_snm.npz"), index=idx_snm.astype(np.int32),
                        dist=dist.astype(np.float64))
    print("snm", idx_snm[:10])

    q_sam = rom.slicing_and_match(ac.copy(), slices_, ppr, pdr, ref_orientations=quats)
    idx_sam = np.array([np.flatnonzero((quats == q).all(axis=1))[0] for q in q_sam])
    np.savez_compressed(os.path.join(HERE, "golden_sam.npz"), index=idx_sam.astype(np.int32))
    print("sam", idx_sam[:10])

    # --- forward / adjoint glue ---------------------------------------------
    import spinifel.autocorrelation as rac

    o = cases.OPS
    ugrid, sup, H_, K_, L_, nuv = cases.ops_inputs()
    fwd = rac.forward(ugrid.copy(), H_, K_, L_, sup, True, H_.size)
    adj = rac.adjoint(nuv, H_, K_, L_, o["M"], True, sup)
    np.savez_compressed(os.path.join(HERE, "golden_ops.npz"), forward=fwd, adjoint=adj)
    print("ops", fwd[:3], adj.ravel()[:3])

    # --- Merge.solve_ac --------------------------------------------------------
    g = cases.MERGE
    sys.argv = ["spinifel", "--mode=sequential", "--settings=" + _settings_file(
        {"det_shape": g["det_shape"], "n_orient": 10, "batch": 10, "maxiter": g["maxiter"]})]
    st._SpinifelSettings__toml = sys.argv[2].split("=", 1)[1]
    st.refresh()
    st._M_override = g["M"]
    import spinifel.sequential.autocorrelation as rsac

    # Merge reads settings.M / M_ups (Mquat-derived); patch the properties for
    # the small test grid
    type(st).M = property(lambda self: g["M"])
    type(st).M_ups = property(lambda self: 2 * g["M"])
    orig_cg = rsac.cg

    def cg_get(*a, **k):
        x, info = orig_cg(*a, **k)
        return x.view(_GetArray), info

    rsac.cg = cg_get
    data, ppr, pdr, orient, ac_est = cases.merge_inputs()
    mquats = orient
    nufft_m = OracleNUFFT(mquats, ppr, pdr)
    merge = rsac.Merge(st, data, ppr, pdr, nufft_m)
    ac_out = merge.solve_ac(0, orient, ac_est.copy())
    np.savez_compressed(os.path.join(HERE, "golden_merge.npz"), ac=ac_out,
                        iterations=np.array(merge.callback.counter))
    print("merge", ac_out.ravel()[:4], merge.callback.counter)


    # --- phasing.phase -----------------------------------------------------------
    p = cases.PHASE
    sys.argv = ["spinifel", "--mode=sequential", "--settings=" + _settings_file(
        {"det_shape": (1, 1, 1), "n_orient": 10, "batch": 10,
         "extra": f"nER = {p['nER']}\nnHIO = {p['nHIO']}\nN_phase_loops = "
                  f"{p['N_phase_loops']}\nbeta = {p['beta']}\n"})]
    st._SpinifelSettings__toml = sys.argv[2].split("=", 1)[1]
    st.refresh()
    type(st).Mquat = property(lambda self: p["Mquat"])
    if not hasattr(np, "infty"):
        np.infty = np.inf
    import spinifel.sequential.phasing as rph

    ac, rho0 = cases.phase_inputs()
    ac_phased, support_, rho_ = rph.phase(0, ac.copy(), None, rho0.copy())
    np.savez_compressed(os.path.join(HERE, "golden_phase.npz"), ac_phased=ac_phased,
                        support_=np.asarray(support_, dtype=np.uint8), rho_=rho_)
    print("phase", ac_phased.ravel()[:3], int(np.asarray(support_).sum()))


    # --- prep: clipping and binning ------------------------------------------------
    pr = _prep_golden()
    np.savez_compressed(os.path.join(HERE, "golden_prep.npz"), **pr)
    print("prep", {k: v.shape for k, v in pr.items()})

    # --- eval: FSC and alignment -------------------------------------------------
    ev = _eval_golden()
    np.savez_compressed(os.path.join(HERE, "golden_eval.npz"), **ev)
    print("eval", ev["resolution"], ev["final_cc"])

    # --- MergeMPI: ranks as threads ----------------------------------------------
    sweep = _mpi_merge_sweep(st, g, rsac)
    np.savez_compressed(os.path.join(HERE, "golden_sweep.npz"), **sweep)
    print("sweep", sweep["ref_rank_gen0"], sweep["ref_rank_gen1"], sweep["summary_gen0"][:, 2])


def _prep_golden():
    sys.modules["h5py"] = types.ModuleType("h5py")
    sys.modules.setdefault("mrcfile", types.ModuleType("mrcfile"))
    if not hasattr(np, "int"):
        np.int = int
    import spinifel.prep as rprep

    c = cases.PREP
    f4, f1, index_map, ppr = cases.prep_inputs()
    nc, nb = c["n_clip"], c["n_bin"]
    dist = rprep.compute_pixel_distance(ppr)
    qs, saxs = rprep.get_saxs(dist, f4.mean(axis=0))
    return dict(sum4=rprep.bin2nx2n_sum(rprep.clipping(f4, nc), nb),
                mean4=rprep.bin2nx2n_mean(rprep.clipping(f4, nc), nb),
                sum1=rprep.bin2nx2n_sum(rprep.clipping(f1, nc), nb),
                sum4_noclip=rprep.bin2nx2n_sum(rprep.clipping(f4, 0), nb),
                index4=rprep.bin2nx2n_index(rprep.clipping_index(index_map.copy(), nc), nb),
                dist=dist, saxs_q=qs, saxs=saxs)


def _eval_golden():
    mpl = sys.modules["matplotlib"]
    mpl.use = lambda *a, **k: None
    mrc = types.ModuleType("mrcfile")
    sys.modules["mrcfile"] = mrc
    v1, v2, uniform_quat, random_quat, randn = cases.eval_inputs()
    skp = sys.modules["skopi"]
    skp.get_uniform_quat = lambda n, avoid_symmetric=True: uniform_quat(n)
    skp.get_random_quat = lambda n: random_quat(n)
    import eval.align as ral
    import eval.fsc as rfsc

    c = cases.EVAL
    res, rshell, fsc = rfsc.compute_fsc(v1, v2, c["dmax"], spacing=c["spacing"])
    quats = uniform_quat(12)
    rot = ral.rotate_volume(v1, quats[:3])
    ccs = ral.score_deformations(v1, v2, quats)
    cen = ral.center_volume(v2)
    np.random.seed(c["seed"] + 2)  # the search's randn draws
    r_vol, m2, final_cc = ral.align_volumes(v1, v2, n_iterations=c["n_iterations"],
                                            n_search=c["n_search"])
    return dict(resolution=np.array(res), rshell=rshell, fsc=fsc, quats=quats, rot=rot,
                ccs=ccs, centred=cen, r_vol=r_vol, mrc2=m2, final_cc=np.array(final_cc))


class _ThreadComm:
    """An in-process stand-in for an MPI communicator whose ranks are
    threads: gather / bcast / Bcast through a barrier."""

    def __init__(self, size):
        import threading

        self.size = size
        self._bar = threading.Barrier(size)
        self._slots = [None] * size
        self._local = threading.local()
        self._data = None

    @property
    def rank(self):
        return self._local.rank

    def gather(self, obj, root=0):
        self._slots[self.rank] = obj
        self._bar.wait()
        out = list(self._slots) if self.rank == root else None
        if out is not None:
            self.last_gather = out
        self._bar.wait()
        return out

    def bcast(self, obj, root=0):
        if self.rank == root:
            self._data = obj
        self._bar.wait()
        out = self._data
        self._bar.wait()
        return out

    def Bcast(self, buf, root=0):
        if self.rank == root:
            self._data = np.array(buf, copy=True)
        self._bar.wait()
        buf[...] = self._data
        self._bar.wait()


def _mpi_merge_sweep(st, g, rsac):
    import threading

    size = cases.SWEEP["size"]
    comm = _ThreadComm(size)
    ctx = types.ModuleType("spinifel.contexts")
    ctx.comm_compute = comm
    sys.modules["spinifel.contexts"] = ctx
    import spinifel
    spinifel.contexts = ctx
    mpi4py = types.ModuleType("mpi4py")
    mpi4py.MPI = types.SimpleNamespace(COMM_WORLD=comm)
    sys.modules["mpi4py"] = mpi4py
    mpi_pkg = types.ModuleType("spinifel.mpi")
    mpi_pkg.__path__ = [os.path.join(REF, "spinifel", "mpi")]
    sys.modules["spinifel.mpi"] = mpi_pkg
    import spinifel.mpi.autocorrelation as rmac

    data, ppr, pdr, orient, ac_est = cases.merge_inputs()
    out = {}
    for gen, est in ((0, None), (1, ac_est)):
        res = [None] * size
        merges = [None] * size

        def run(rank):
            comm._local.rank = rank
            m = rmac.MergeMPI(st, data, ppr, pdr, OracleNUFFT(orient, ppr, pdr))
            merges[rank] = m
            res[rank] = m.solve_ac(gen, orient, None if est is None else est.copy())

        th = [threading.Thread(target=run, args=(r,)) for r in range(size)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        out[f"ac_gen{gen}"] = np.asarray(res[0].real)
        out[f"ref_rank_gen{gen}"] = np.array(merges[0].ref_rank)
        # (rank, rlambda, ||x||, ||W x - d||) as rank 0 gathered them
        out[f"summary_gen{gen}"] = np.array(comm.last_gather, dtype=np.float64)
        assert all(np.array_equal(res[0], r) for r in res)
    return out


if __name__ == "__main__":
    main()
