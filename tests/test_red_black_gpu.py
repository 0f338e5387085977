"""EquSolver in red-black order (the reference's OpenMP EquSolver) on the GPU.

Pinned two ways: against the reference's own compiled OpenMP EquSolver
(golden vectors: its odd-then-even ids, its uint8 images at every
checkpoint, its err), and bit for bit against the oracle's red-black
restatement (float32 states), including the 640,000-unknown square800
system at 5000 sweeps.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, problem_args
from oracle import cjacobi, np_jacobi
from oracle import prep as oprep

pytestmark = pytest.mark.gpu

OMP_EQU_CASES = ["rand24", "circle256", "avg_offsets", "blob_frame"]


@pytest.fixture(scope="module")
def backend():
    from fpie_gb300 import backend as b

    return b


@pytest.mark.parametrize("name", OMP_EQU_CASES)
def test_partition_matches_reference_openmp(backend, name):
    d = load_golden(name)
    s = backend.EquSolver(1024, order="red_black")
    mc = d["grid_mask"]
    ids = s.partition(mc)
    np.testing.assert_array_equal(np.where(mc > 0, ids, 0), d["omp_equ_ids"])
    _, n_mid = np_jacobi.red_black_ids(mc)
    assert s.n_mid == n_mid and s.order == "red_black"


KERNELS = {"auto": "grid:rb16w8k8", "gather": "red_black", "rb16w8k8": "grid:rb16w8k8",
           "rb16w8k8d": "grid:rb16w8k8d"}


@pytest.mark.parametrize("kernel", sorted(KERNELS))
@pytest.mark.parametrize("name", OMP_EQU_CASES)
def test_states_images_and_err(backend, name, kernel):
    """Grid placement (the packed red-black kernel) and the equation kernels."""
    d = load_golden(name)
    e = oprep.equ_inputs(*problem_args(d), order="red_black")
    s = backend.EquSolver(1024, order="red_black")
    s.set_kernel(kernel)
    s.partition(e["mask"])
    s.reset(e["N"], e["A"], e["X"], e["B"])
    assert s.kernel == KERNELS[kernel]
    o = np_jacobi.EquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    idx = e["tgt_index"]
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    done = 0
    for k in (int(v) for v in d["checkpoints"]):
        img, err = s.step(k - done)
        o.sweep(k - done)
        done = k
        np.testing.assert_array_equal(s.state(), o.X)
        np.testing.assert_array_equal(img, o.image())
        np.testing.assert_array_equal(img[1:], d[f"omp_equ_img_{k}"][idx[0] - x0, idx[1] - y0])
        np.testing.assert_allclose(err, o.err64(), rtol=1e-5)
        np.testing.assert_allclose(err, d[f"omp_equ_err_{k}"], rtol=1e-5, atol=1e-2)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_step_splits_across_graph_chunks(backend, kernel):
    """Uneven steps (remainder sweeps, 64-sweep graph chunks) continue the state."""
    d = load_golden("circle256")
    e = oprep.equ_inputs(*problem_args(d), order="red_black")
    s = backend.EquSolver(256, order="red_black")
    s.set_kernel(kernel)
    s.partition(e["mask"])
    s.reset(e["N"], e["A"], e["X"], e["B"])
    o = cjacobi.CEquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    for k in (3, 64, 130, 1):
        s.step(k)
        o.sweep(k)
        np.testing.assert_array_equal(s.state(), o.X)


@pytest.fixture(scope="module")
def square800_rb():
    from fpie_gb300 import workloads

    pb = workloads.square800()
    e = oprep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient,
                         order="red_black")
    assert e["N"] == 640_001
    o = cjacobi.CEquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    o.sweep(5000)
    return e, o


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_square800_5000_sweeps(backend, square800_rb, kernel):
    e, o = square800_rb
    s = backend.EquSolver(1024, order="red_black")
    s.set_kernel(kernel)
    s.partition(e["mask"])
    s.reset(e["N"], e["A"], e["X"], e["B"])
    assert s.kernel == KERNELS[kernel]
    img, err = s.step(5000)
    np.testing.assert_array_equal(s.state(), o.X)
    np.testing.assert_array_equal(img, o.image())
    np.testing.assert_allclose(err, o.err64(), rtol=1e-5)


def test_components_and_parity_shift(backend):
    """Several components (the placement stacks them and shifts a component
    one column where its colouring needs it): grid placement equals the
    oracle bit for bit."""
    rng = np.random.default_rng(11)
    mask = np.zeros((60, 70), np.uint8)
    mask[3:20, 4:30] = 255
    mask[25:40, 35:66] = 255
    mask[44:57, 9:12] = 255
    mask[44:50, 20:21] = 255
    src = rng.integers(0, 256, size=(60, 70, 3), dtype=np.uint8)
    tgt = rng.integers(0, 256, size=(60, 70, 3), dtype=np.uint8)
    e = oprep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), "max", order="red_black")
    s = backend.EquSolver(256, order="red_black")
    s.partition(e["mask"])
    s.reset(e["N"], e["A"], e["X"], e["B"])
    assert s.kernel == "grid:rb16w8k8"
    s.step(77)
    o = np_jacobi.EquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    o.sweep(77)
    np.testing.assert_array_equal(s.state(), o.X)


def test_non_raster_system_runs_on_the_equation_kernels(backend):
    """A coloured system that is not a raster stencil (one link dropped on
    both sides) falls back to the equation kernels, still exact."""
    d = load_golden("circle256")
    e = oprep.equ_inputs(*problem_args(d), order="red_black")
    A = e["A"].copy()
    i = int(np.nonzero(A[1:, 3])[0][0]) + 1  # a row with a right neighbour
    j = int(A[i, 3])
    A[i, 3] = 0
    A[j, 2] = 0
    s = backend.EquSolver(256, order="red_black")
    s.partition(e["mask"])
    s.reset(e["N"], A, e["X"], e["B"])
    assert s.kernel == "red_black"
    s.step(70)
    o = np_jacobi.EquRedBlack(A, e["X"], e["B"], e["n_mid"])
    o.sweep(70)
    np.testing.assert_array_equal(s.state(), o.X)


def test_grid_kernel_names_refused(backend):
    e = oprep.equ_inputs(*problem_args(load_golden("rand24")), order="red_black")
    s = backend.EquSolver(1024, order="red_black")
    s.set_kernel("p16w8k16")
    s.partition(e["mask"])
    with pytest.raises(ValueError):
        s.reset(e["N"], e["A"], e["X"], e["B"])
    g = backend.GridSolver(8, 8)
    with pytest.raises(ValueError):
        g.set_kernel("rb16w8k8")  # not a Jacobi kernel


def test_refuses_a_system_of_the_wrong_colouring(backend):
    d = load_golden("rand24")
    s = backend.EquSolver(1024, order="red_black")
    s.partition(d["grid_mask"])
    # The numpy backend's row-major system: neighbours of one colour collide.
    with pytest.raises(ValueError, match="colour"):
        s.reset(int(d["equ_N"]), d["equ_A"], d["equ_X"], d["equ_B"])


def test_refuses_reset_without_partition(backend):
    e = oprep.equ_inputs(*problem_args(load_golden("rand24")), order="red_black")
    s = backend.EquSolver(1024, order="red_black")
    with pytest.raises(RuntimeError, match="partition"):
        s.reset(e["N"], e["A"], e["X"], e["B"])


def test_order_change_discards_the_system(backend):
    e = oprep.equ_inputs(*problem_args(load_golden("rand24")), order="red_black")
    s = backend.EquSolver(1024, order="red_black")
    s.partition(e["mask"])
    s.reset(e["N"], e["A"], e["X"], e["B"])
    s.step(3)
    s.set_order("jacobi")
    assert s.order == "jacobi"
    with pytest.raises(RuntimeError):
        s.sweeps(1)
    ids = s.partition(e["mask"])  # row-major again
    np.testing.assert_array_equal(ids[e["mask"] > 0], np.arange(1, int((e["mask"] > 0).sum()) + 1))


@pytest.mark.parametrize("name", OMP_EQU_CASES)
def test_reset_images_numbers_red_black(backend, name):
    """The GPU-side reset from the uint8 images builds the red-black system:
    the OpenMP partition's numbering, the host reset's A / B, and the same
    sweeps."""
    d = load_golden(name)
    src, mask, tgt, mos, mot, grad = problem_args(d)
    e = oprep.equ_inputs(src, mask, tgt, mos, mot, grad, order="red_black")
    s = backend.EquSolver(1024, order="red_black")
    N, box, (rows, cols) = s.reset_images(src, mask, tgt, mos, mot, grad)
    assert N == e["N"] and s.n_mid == e["n_mid"]
    A, B = s.inputs()
    np.testing.assert_array_equal(A, e["A"])
    np.testing.assert_array_equal(B, e["B"])
    np.testing.assert_array_equal(rows, e["tgt_index"][0])
    np.testing.assert_array_equal(cols, e["tgt_index"][1])
    s.step(37)
    o = np_jacobi.EquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    o.sweep(37)
    np.testing.assert_array_equal(s.state(), o.X)


@pytest.mark.parametrize("name", ["circle256", "blob_frame"])
@pytest.mark.parametrize("device_prep", [False, True])
def test_processor_matches_reference_openmp(name, device_prep):
    """EquProcessor(backend='gb300-rb') end to end, host or GPU-side reset,
    equals the reference's OpenMP EquProcessor's merged images (the golden
    crop)."""
    from fpie_gb300 import process

    d = load_golden(name)
    src, mask, tgt, mos, mot, grad = problem_args(d)
    p = process.EquProcessor(gradient=grad, backend="gb300-rb", device_prep=device_prep)
    p.reset(src, mask, tgt, mos, mot)
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    done = 0
    for k in (int(v) for v in d["checkpoints"]):
        img, err = p.step(k - done)
        done = k
        np.testing.assert_array_equal(img[x0:x1, y0:y1], d[f"omp_equ_img_{k}"])
        np.testing.assert_allclose(err, d[f"omp_equ_err_{k}"], rtol=1e-5, atol=1e-2)


def test_order_arguments_checked(backend):
    from fpie_gb300 import _abi

    s = backend.EquSolver(256)
    with pytest.raises(ValueError):
        s.set_order("gauss")
    with pytest.raises(_abi.FpieArgumentError):
        _abi.call("fpie_equ_set_order", s._h, 7)
    assert s.order == "jacobi" and s.n_mid == 0


def test_placed_reset_in_red_black_order(backend):
    from fpie_gb300 import prep as pprep

    d = load_golden("blob_frame")
    src, mask, tgt, mos, mot, grad = problem_args(d)
    s = backend.EquSolver(1024, order="red_black")
    sysm = pprep.equ_inputs(src, mask, tgt, mos, mot, grad, s.partition)
    s.reset(sysm.N, sysm.A, sysm.X, sysm.B, placement=sysm.placement())
    assert s.kernel == "grid:rb16w8k8"
    s.step(33)
    o = np_jacobi.EquRedBlack(sysm.A, sysm.X, sysm.B, s.n_mid)
    o.sweep(33)
    np.testing.assert_array_equal(s.state(), o.X)
    # the colours must sit on their parity: a placement shifted by one column is refused
    pos, n, m = sysm.placement()
    shifted = pos.copy()
    shifted[1:] = (pos[1:] // m) * (m + 1) + pos[1:] % m + 1  # one column right: parity flips
    t = backend.EquSolver(1024, order="red_black")
    t.partition(d["grid_mask"])
    with pytest.raises(ValueError):
        t.reset(sysm.N, sysm.A, sysm.X, sysm.B, placement=(shifted, n, m + 1))
    # the same shift is a valid placement for the Jacobi order (no colouring)
    j = backend.EquSolver(1024)
    jsys = pprep.equ_inputs(src, mask, tgt, mos, mot, grad, j.partition)
    jpos, jn, jm = jsys.placement()
    jshift = jpos.copy()
    jshift[1:] = (jpos[1:] // jm) * (jm + 1) + jpos[1:] % jm + 1
    j.reset(jsys.N, jsys.A, jsys.X, jsys.B, placement=(jshift, jn, jm + 1))
    assert j.kernel.startswith("grid:")
