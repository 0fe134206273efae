"""C-ABI checks that need no GPU: the library loads, exports every symbol that
include/qf.h declares, and its host-only logic (validation, planning,
SmallRng jump-ahead) behaves."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from quantumforge_gb300 import _abi as A
from quantumforge_gb300 import _native
from quantumforge_gb300 import workloads as W

HEADER = Path(__file__).resolve().parent.parent / "include" / "qf.h"


def header_functions():
    """Functions the library exports: declarations, not the header-only
    `static inline` helpers."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"static inline[^{]*\{.*?\n\}", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qf_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_signatures():
    decl = header_functions()
    assert decl, "no declarations parsed"
    assert set(decl) == set(_native.SIGNATURES), set(decl) ^ set(_native.SIGNATURES)


def test_library_exports_every_header_symbol(engine_lib):
    lib = C.CDLL(str(_native.lib_path()))
    for name in header_functions():
        assert hasattr(lib, name), f"{name} missing from {_native.lib_path().name}"


def test_abi_version_and_status_names(engine_lib):
    assert engine_lib.qf_abi_version() == 1
    for code, name in A.STATUS_NAMES.items():
        got = engine_lib.qf_status_name(code).decode()
        expect = "QF_OK" if code == 0 else "QF_ERR_" + re.sub(r"(?<!^)(?=[A-Z])", "_", name).upper()
        assert got == expect, (code, got, expect)


def test_struct_layouts_match_header():
    assert C.sizeof(A.Op) == 24 and A.OP_DTYPE.itemsize == 24
    assert C.sizeof(A.PauliTerm) == 32
    assert A.Op.theta.offset == 16 and A.Op.param.offset == 12
    assert C.sizeof(A.ExecOpts) == 16
    assert C.sizeof(A.GradientOpts) == 48


def test_channel_aux_encoding_matches_the_header_helpers(tmp_path):
    """channel_record's (q1, param) split equals qf_op_set_aux / qf_op_aux."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "aux.c"
    src.write_text('#include "qf.h"\n'
                   "double get_aux(const qf_op *op) { return qf_op_aux(op); }\n"
                   "void set_aux(qf_op *op, double v) { qf_op_set_aux(op, v); }\n")
    so = tmp_path / "libaux.so"
    subprocess.run([cc, "-shared", "-fPIC", f"-I{HEADER.parent}", str(src), "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    lib.get_aux.restype = C.c_double
    lib.get_aux.argtypes = [C.c_void_p]
    lib.set_aux.argtypes = [C.c_void_p, C.c_double]
    for beta in (0.0, 0.7, 1.0, 123.456, 1e-300, float("inf")):
        rec = A.ops_array([A.channel_record(A.CHANNEL_THERMAL_DAMPING, 3, 0.2, beta)])
        assert lib.get_aux(rec.ctypes.data) == beta
        other = A.ops_array([(A.OP_CHANNEL, A.CHANNEL_THERMAL_DAMPING, 3, 0, 0, 0.2)])
        lib.set_aux(other.ctypes.data, beta)
        assert other.tobytes() == rec.tobytes()


@pytest.mark.parametrize("seed,steps", [(0, 0), (1, 1), (42, 7), (721, 64), (991, 1000), (1234, 123457)])
def test_rng_jump_equals_stepping(engine_lib, seed, steps):
    r = O.Rng(seed)
    start = r.state.value
    for _ in range(steps):
        r.next_u64()
    assert engine_lib.qf_rng_jump(start, steps) == r.state.value


def plan_stats(engine_lib, n, ops, params=None, tile=0, mode=A.EXEC_AUTO, dtype=A.C64):
    p = None if params is None else np.ascontiguousarray(params, dtype=np.float64)
    npass, ngate = C.c_uint64(), C.c_uint64()
    o = A.ExecOpts(mode, tile, 0, 0)
    st = engine_lib.qf_plan_stats(n, dtype, _native.ptr(ops), len(ops), _native.ptr(p), 0 if p is None else p.size,
                                  None, 0, C.byref(o), C.byref(npass), C.byref(ngate))
    return st, npass.value, ngate.value


def test_plan_fuses_a_random_circuit(engine_lib):
    ops = W.random_circuit(30, 40, 1, two_qubit="mixed")
    st, npass, ngate = plan_stats(engine_lib, 30, ops)
    assert st == 0 and ngate == len(ops)
    st, unf, _ = plan_stats(engine_lib, 30, ops, mode=A.EXEC_UNFUSED)
    assert unf == ngate
    assert npass * 8 < ngate, (npass, ngate)
    # wider tiles never need more passes
    counts = [plan_stats(engine_lib, 30, ops, tile=k)[1] for k in (8, 10, 12, 14)]
    assert counts == sorted(counts, reverse=True), counts


def test_lookahead_residency_needs_fewer_passes_than_first_come(engine_lib):
    """The 30-qubit depth-40 headline circuit on 12-qubit tiles: 47 passes when
    each pass's resident qubits are chosen by look-ahead (greedy rollouts), 74
    first-come."""
    ops = W.random_circuit(30, 40, 1, two_qubit="mixed")
    npass = C.c_uint64()
    counts = {}
    for flags, name in ((0, "lookahead"), (A.EXEC_FLAG_PLAN_FIRST_COME, "first_come")):
        o = A.ExecOpts(A.EXEC_AUTO, 12, 0, flags)
        ng = C.c_uint64()
        assert engine_lib.qf_plan_stats(30, A.C64, _native.ptr(ops), len(ops), None, 0, None, 0, C.byref(o),
                                        C.byref(npass), C.byref(ng)) == 0
        counts[name] = npass.value
    assert counts == {"lookahead": 47, "first_come": 74}
    for seed in (2, 3):
        ops = W.random_circuit(26, 30, seed, two_qubit="mixed")
        la = plan_stats(engine_lib, 26, ops)[1]
        o = A.ExecOpts(A.EXEC_AUTO, 0, 0, A.EXEC_FLAG_PLAN_FIRST_COME)
        ng = C.c_uint64()
        engine_lib.qf_plan_stats(26, A.C64, _native.ptr(ops), len(ops), None, 0, None, 0, C.byref(o), C.byref(npass),
                                 C.byref(ng))
        assert la < npass.value, (seed, la, npass.value)


def test_plan_small_state_is_one_pass(engine_lib):
    ops = W.random_circuit(10, 20, 3, two_qubit="mixed")
    st, npass, _ = plan_stats(engine_lib, 10, ops)
    assert st == 0 and npass == 1


def test_plan_diagonal_gates_need_no_residency(engine_lib):
    # Rz and CZ on high qubits never force a new pass
    recs = [(A.OP_GATE, A.GATE_RZ, q, 0, 0, 0.1 * q) for q in range(30)]
    recs += [(A.OP_CZ, 0, q, 29 - q, 0, 0.0) for q in range(15)]
    st, npass, _ = plan_stats(engine_lib, 30, A.ops_array(recs))
    assert st == 0 and npass == 1


@pytest.mark.parametrize(
    "recs,params,kind",
    [
        ([(A.OP_GATE, A.GATE_H, 5, 0, 0, 0.0)], None, "QubitOutOfRange"),
        ([(A.OP_CNOT, 0, 1, 1, 0, 0.0)], None, "InvalidQubitPair"),
        ([(A.OP_CZ, 0, 0, 9, 0, 0.0)], None, "QubitOutOfRange"),
        ([(A.OP_CHANNEL, 0, 0, 0, 0, 0.0)], None, "OperationRequiresDensityMatrix"),
        ([(A.OP_MEASURE, 0, 0, 0, 0, 0.0)], None, "OperationRequiresShotExecution"),
        ([(A.OP_ROTATION, A.PAULI_Y, 0, 0, 3, 0.0)], [0.1], "InvalidParameterCount"),
        ([(A.OP_ROTATION, A.PAULI_Y, 0, 0, 0, 0.0)], [float("nan")], "NonFiniteParameter"),
        ([(A.OP_GATE, 42, 0, 0, 0, 0.0)], None, "InvalidArgument"),
    ],
)
def test_plan_validation_errors(engine_lib, recs, params, kind):
    st, _, _ = plan_stats(engine_lib, 3, A.ops_array(recs), params=params)
    assert A.STATUS_NAMES[st] == kind
    assert engine_lib.qf_last_error().decode()


def test_zero_qubits_rejected(engine_lib):
    st, _, _ = plan_stats(engine_lib, 0, A.ops_array([]))
    assert A.STATUS_NAMES[st] == "ZeroQubits"


def test_context_creation_reports_missing_gpu_cleanly(engine_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible; covered by the gpu tests")
    h = C.c_void_p()
    st = engine_lib.qf_ctx_create(0, C.byref(h))
    assert A.STATUS_NAMES[st] == "Cuda" and not h.value


def _block_plan(engine_lib, n, ops, k, dtype=A.C64, flags=0):
    npass, ngate = C.c_uint64(), C.c_uint64()
    o = A.ExecOpts(A.EXEC_AUTO, 0, k, flags)
    st = engine_lib.qf_plan_stats(n, dtype, _native.ptr(ops), len(ops), None, 0, None, 0, C.byref(o), C.byref(npass),
                                  C.byref(ngate))
    return st, npass.value


@pytest.mark.parametrize("dtype", [A.C64, A.C128])
def test_dense_block_plans(engine_lib, dtype):
    """k-qubit block fusion plans every width 2..5 (every touched qubit is then
    tile-resident, so a block plan never has fewer passes than the plain one
    on the same tiles), and rejects widths outside 0..5."""
    ops = W.random_circuit(30, 40, 1, two_qubit="mixed")
    st, plain = _block_plan(engine_lib, 30, ops, 0, dtype)
    assert st == 0
    for k in (2, 3, 4, 5):
        st, npass = _block_plan(engine_lib, 30, ops, k, dtype)
        assert st == 0 and npass >= plain, (k, npass, plain)
        assert npass * 8 < len(ops)
    assert _block_plan(engine_lib, 30, ops, 1, dtype) == (0, plain)  # width 1: gates one by one
    for bad in (6, -1):
        st, _ = _block_plan(engine_lib, 30, ops, bad, dtype)
        assert A.STATUS_NAMES[st] == "InvalidArgument"
    # a small state is one pass whatever the width
    small = W.random_circuit(4, 6, 2, two_qubit="mixed")
    assert _block_plan(engine_lib, 4, small, 5, dtype) == (0, 1)


def test_adjoint_plan_stats(engine_lib):
    """Launch counts and algorithmic bytes of one adjoint gradient (host only):
    a checkpoint per layer adds state copies and never removes passes."""
    ops, params, H = W.vqe_tfim(24, 8, seed=3)
    t = H.array()
    out = {}
    for every in (0, 72):
        o = A.GradientOpts()
        o.strategy, o.dtype, o.checkpoint_every = A.GRAD_ADJOINT, A.C64, every
        st = A.AdjointStats()
        p = np.ascontiguousarray(params, dtype=np.float64)
        assert engine_lib.qf_adjoint_plan_stats(24, A.C64, _native.ptr(ops), len(ops), _native.ptr(p), p.size, None, 0,
                                                _native.ptr(t), len(t), C.byref(o), C.byref(st)) == 0
        out[every] = st
        N = (1 << 24) * 8
        assert st.forward_passes >= 1 and st.backward_passes >= 1 and st.pauli_passes >= 1
        assert st.hbm_bytes >= N * (1 + 2 * st.forward_passes + 4 * st.backward_passes + 2)
    assert out[0].state_copies == 0 and out[72].state_copies == 2 * (8 - 1)
    assert out[72].forward_passes >= out[0].forward_passes
