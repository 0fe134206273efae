"""Circuit formats through the C ABI (host code, no GPU): OpenQASM 2.0 import,
QASM export and the JSON form, against the reference's own tests
(src/qasm.rs:1076-1253, tests/qasm_parse_test.rs, src/qasm_export.rs tests,
src/serialize.rs tests, tests/module_coverage.rs:19-35) and against the
oracle for what the parsed circuits compute."""
import json
import math

import numpy as np
import pytest

import oracle as O
import quantumforge_gb300 as qf
from quantumforge_gb300 import _abi as A
from quantumforge_gb300.core import NoiseChannel, parse_qasm_ops

H = 'OPENQASM 2.0;\ninclude "qelib1.inc";\n'


def n_ops(src):
    return len(qf.parse_qasm(src).operations)


def err(src):
    with pytest.raises(qf.QuantumError) as e:
        qf.parse_qasm(src)
    return str(e.value)


# ---- src/qasm.rs unit tests -----------------------------------------------------
def test_parse_simple_bell():
    assert n_ops('\nOPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2];\ncreg c[2];\nh q[0];\ncx q[0], q[1];\n'
                 'measure q[0] -> c[0];\n') == 3


def test_parse_single_qubit_gates():
    src = "\nOPENQASM 2.0;\nqreg q[1];\n" + "".join(f"{g} q[0];\n" for g in ("x", "y", "z", "h", "s", "sdg", "t", "tdg"))
    ops = parse_qasm_ops(src)[0]
    assert len(ops) == 8
    assert list(ops["gate"]) == [A.GATE_X, A.GATE_Y, A.GATE_Z, A.GATE_H, A.GATE_S, A.GATE_SDG, A.GATE_T, A.GATE_TDG]


def test_parse_parameterized_gates():
    ops = parse_qasm_ops("\nOPENQASM 2.0;\nqreg q[1];\nrx(3.14159) q[0];\nry(1.5708) q[0];\nrz(0.7854) q[0];\n")[0]
    assert list(ops["gate"]) == [A.GATE_RX, A.GATE_RY, A.GATE_RZ]
    assert list(ops["theta"]) == [3.14159, 1.5708, 0.7854]


def test_parse_u_gates():  # u1 -> Rz; u2, u3 -> Rz Ry Rz
    ops = parse_qasm_ops("\nOPENQASM 2.0;\nqreg q[1];\nu1(0.5) q[0];\nu2(0.3, 0.7) q[0];\nu3(0.1, 0.2, 0.3) q[0];\n")[0]
    assert len(ops) == 7
    assert [(int(o["gate"]), float(o["theta"])) for o in ops] == [
        (A.GATE_RZ, 0.5), (A.GATE_RZ, 0.3), (A.GATE_RY, math.pi / 2), (A.GATE_RZ, 0.7),
        (A.GATE_RZ, 0.2), (A.GATE_RY, 0.1), (A.GATE_RZ, 0.3)]


def test_parse_toffoli_is_the_15_op_decomposition_of_ccx():
    ops = parse_qasm_ops("\nOPENQASM 2.0;\nqreg q[3];\nccx q[0], q[1], q[2];\n")[0]
    assert len(ops) == 15
    for basis in range(8):  # the decomposition is Toffoli exactly (no global phase)
        a = np.zeros(8, complex)
        a[basis] = 1
        out = O.run(ops, 3, init=a)
        want = basis ^ 4 if (basis & 3) == 3 else basis
        assert abs(out[want] - 1) < 1e-12 and np.abs(np.delete(out, want)).max() < 1e-12


def test_parse_multiple_registers():
    ops = parse_qasm_ops("\nOPENQASM 2.0;\nqreg a[2];\nqreg b[2];\ncx a[0], b[1];\n")[0]
    assert len(ops) == 1 and (int(ops[0]["q0"]), int(ops[0]["q1"])) == (0, 3)


def test_parse_gate_definition():
    assert n_ops("\nOPENQASM 2.0;\nqreg q[2];\ngate mygate a, b {\n    h a;\n    cx a, b;\n}\nmygate q[0], q[1];\n") == 2


def test_barrier_is_a_no_op_and_reset_is_rejected():
    msg = err("\nOPENQASM 2.0;\nqreg q[2];\nh q[0];\nbarrier q;\nreset q[0];\ncx q[0], q[1];\n")
    assert "line 6" in msg and "reset is not supported" in msg
    assert n_ops(H + "qreg q[2];\nh q[0];\nbarrier q;\ncx q[0], q[1];\n") == 2


@pytest.mark.parametrize("src,needle", [
    ("\nOPENQASM 3.0;\nqubit q;\n", "unknown qubit register 'q'"),
    ("\nqreg q[1];\nh q[0];\n", "missing OPENQASM 2.0 header"),
    ("\nOPENQASM 2.0;\nqreg q[1];\nfoo q[0];\n", "unknown gate 'foo'"),
    ("\nOPENQASM 2.0;\nqreg q[1];\nh q[5];\n", "qubit index 5 out of range for register 'q' (size 1)"),
    ("\nOPENQASM 2.0;\nqreg q[1];\nrx(pi/0) q[0];\n", "invalid parameter 'pi/0'"),
    ("\nOPENQASM 2.0;\nqreg q[1];\ncreg c[1];\nmeasure q[0] c[0];\n", "measure requires 'q[i] -> c[j]'"),
    ("\nOPENQASM 2.0;\nqreg q[1];\nh r[0];\n", "unknown qubit register 'r'"),
    ("\nOPENQASM 2.0;\nqreg q[2];\ngate g a {\n h a;\n", "unclosed gate definition"),
])
def test_rejections(src, needle):
    assert needle in err(src)


def test_pi_expressions():
    ops = parse_qasm_ops("\nOPENQASM 2.0;\nqreg q[1];\nrx(pi/2) q[0];\nry(2*pi/3) q[0];\nrz(-pi*0.5+1) q[0];\n")[0]
    assert list(ops["theta"]) == [math.pi / 2, 2 * math.pi / 3, -math.pi * 0.5 + 1]
    # parameters end at the first ')', so nested parentheses do not parse (as in the reference)
    assert "invalid parameter '-(pi+1'" in err(H + "qreg q[1];\nrz(-(pi+1)*0.5) q[0];\n")


def test_the_e_substitution_reads_exponents_as_the_reference_does():
    # `e` is replaced by the digits of E before tokenising: 1e-3 reads 1 2.718... - 3
    ops = parse_qasm_ops(H + "qreg q[1];\nrz(1e-3) q[0];\n")[0]
    assert float(ops[0]["theta"]) == 12.718281828459045 - 3


# ---- tests/qasm_parse_test.rs ---------------------------------------------------
def test_ghz_circuit_runs_normalised():
    src = H + "qreg q[4];\ncreg c[4];\nh q[0];\n" + "".join(f"cx q[{i}], q[{i + 1}];\n" for i in range(3))
    a = O.run(qf.parse_qasm(src).ops(), 4)
    assert abs(np.vdot(a, a).real - 1) < 1e-10
    assert abs(abs(a[0]) ** 2 - 0.5) < 1e-12 and abs(abs(a[15]) ** 2 - 0.5) < 1e-12


def test_statements_sharing_a_line_are_all_parsed():
    shared = qf.parse_qasm(H + "qreg q[2];\nh q[0];cx q[0],q[1];x q[1];\n")
    split = qf.parse_qasm(H + "qreg q[2];\nh q[0];\ncx q[0],q[1];\nx q[1];\n")
    assert len(shared.operations) == 3
    assert shared.to_json() == split.to_json()
    p = O.probabilities(O.run(shared.ops(), 2))
    assert abs(p[1] - 0.5) < 1e-9 and abs(p[2] - 0.5) < 1e-9


def test_trailing_comment_after_a_shared_statement_is_ignored():
    assert n_ops(H + "qreg q[2];\nh q[0]; cx q[0],q[1]; // entangle\n") == 2


def test_multiline_gate_definition_is_left_intact():
    ops = parse_qasm_ops(H + "qreg q[1];\ngate mygate a {\n  x a;\n  h a;\n}\nmygate q[0];\n")[0]
    assert list(ops["gate"]) == [A.GATE_X, A.GATE_H]


def test_user_gate_parameters_and_registers():
    src = H + "qreg q[2];\ngate rot(theta, phi) a, b {\n  rz(theta) a;\n  cx a, b;\n  ry(phi) b;\n  rx(0.25) a;\n}\nrot(0.5, 1.5) q[1], q[0];\n"
    ops, nq, nc = parse_qasm_ops(src)
    assert nq == 2 and nc == 0
    assert [(int(o["kind"]), int(o["gate"]), int(o["q0"]), float(o["theta"])) for o in ops] == [
        (A.OP_GATE, A.GATE_RZ, 1, 0.5), (A.OP_CNOT, 0, 1, 0.0), (A.OP_GATE, A.GATE_RY, 0, 1.5), (A.OP_GATE, A.GATE_RX, 1, 0.25)]


# ---- QASM export (src/qasm_export.rs tests) ---------------------------------------
BELL = "\nOPENQASM 2.0;\ninclude \"qelib1.inc\";\nqreg q[2];\ncreg c[2];\nh q[0];\ncx q[0], q[1];\nmeasure q[0] -> c[0];\nmeasure q[1] -> c[1];\n"


def test_export_simple_bell_and_round_trip():
    c = qf.parse_qasm(BELL)
    out = qf.export_qasm(c)
    for s in ("OPENQASM 2.0", "qreg q[2]", "creg c[2]", "h q[0]", "cx q[0], q[1]", "measure q[0] -> c[0]"):
        assert s in out
    assert len(qf.parse_qasm(out).operations) == len(c.operations)


def test_export_gates_angles_and_swap():
    c = qf.Circuit()
    c.push(qf.Gate.H, 0)
    c.push(qf.Gate.H, 1)
    c.cnot(0, 1)
    c.cz(1, 0)
    c.swap(0, 1)
    c.push(qf.Gate.Rx(math.pi / 2), 0)
    c.push(qf.Gate.Rz(math.pi), 1)
    c.push(qf.Gate.Ry(0.123456789012345), 0)
    out = qf.export_qasm(c)
    assert "cz q[1], q[0]" in out and out.count("cx ") == 4 and "swap " not in out
    assert "rx(pi/2) q[0];" in out and "rz(pi) q[1];" in out and "ry(0.123456789) q[0];" in out
    back = qf.parse_qasm(out)
    assert np.abs(O.run(back.ops(), 2) - O.run(c.ops(), 2)).max() < 1e-9


def test_export_retains_declared_idle_qubits():
    c = qf.Circuit()
    c.push(qf.Gate.H, 0)
    assert "qreg q[4];" in qf.export_qasm_with_qubits(c, 4)
    with pytest.raises(qf.QuantumError) as e:
        qf.export_qasm_with_qubits(c, 0)
    assert "circuit uses a qubit outside the declared register" in str(e.value)


@pytest.mark.parametrize("angle,text", [(0.0, "0"), (math.pi, "pi"), (-math.pi, "-pi"), (math.pi / 2, "pi/2"),
                                        (-math.pi / 2, "-pi/2"), (math.pi / 4, "pi/4"), (0.5, "0.5"), (-1.25, "-1.25")])
def test_format_angle(angle, text):
    c = qf.Circuit()
    c.push(qf.Gate.Rz(angle), 0)
    assert f"rz({text}) q[0];" in qf.export_qasm(c)


def test_export_conditionals_and_channels():
    c = qf.Circuit()
    c.push(qf.Gate.H, 0)
    c.measure(0, 0)
    c.if_classical_bit(0, 1, qf.Gate.X, 1)
    c.channel(1, NoiseChannel.Depolarizing(0.1))
    out = qf.export_qasm(c)
    assert "if (c[0] == 1) x q[1];" in out and "Depolarizing" not in out


# ---- JSON (src/serialize.rs tests, tests/module_coverage.rs:19-35) ----------------
def _full_circuit():
    c = qf.Circuit()
    c.push(qf.Gate.H, 0)
    c.push(qf.Gate.Rx(1.57), 0)
    c.cnot(0, 1)
    c.cz(0, 1)
    c.swap(0, 1)
    c.measure(0, 0)
    c.measure(1, 1)
    c.if_classical_bit(0, 1, qf.Gate.X, 1)
    c.channel(0, NoiseChannel.Depolarizing(0.1))
    c.channel(1, NoiseChannel.AmplitudeDamping(0.05))
    c.channel(1, NoiseChannel.ThermalDamping(0.2, 0.7))
    return c


def test_json_round_trip_and_serde_layout():
    c = _full_circuit()
    text = c.to_json()
    for s in ('"H"', '"cx"', '"measure"', '"conditional"', '"Depolarizing"'):
        assert s in text
    back = qf.Circuit.from_json(text)
    assert back.to_json() == text
    assert qf.Circuit.from_json_bytes(c.to_json_bytes()).ops().tobytes() == c.ops().tobytes()
    doc = json.loads(text)
    assert doc["num_qubits"] == 2 and doc["num_classical_bits"] == 2
    assert doc["operations"][1] == {"type": "single", "gate": "Rx", "target": 0, "params": [1.57]}
    assert doc["operations"][-1] == {"type": "channel", "channel": "ThermalDamping", "target": 1, "params": [0.2, 0.7]}
    assert text.startswith('{\n  "num_qubits": 2,\n  "num_classical_bits": 2,\n  "operations": [\n    {\n      "type": "single",')


@pytest.mark.parametrize("value,text", [(0.0, "0.0"), (1.0, "1.0"), (1.57, "1.57"), (1e-05, "0.00001"), (1e-7, "1e-7"),
                                        (123456789.0, "123456789.0"), (1e17, "1e17"), (-2.5e-9, "-2.5e-9"),
                                        (0.1 + 0.2, "0.30000000000000004"), (1.2345e20, "1.2345e20")])
def test_json_numbers_are_written_like_serde_json(value, text):
    c = qf.Circuit()
    c.push(qf.Gate.Rz(value), 0)
    assert f"\n        {text}\n" in c.to_json()


@pytest.mark.parametrize("doc,needle", [
    ("{ not json", "JSON error"),
    ('{"num_qubits": 1, "operations": []}', "missing field `num_classical_bits`"),
    ('{"num_qubits": 1, "num_classical_bits": 1, "operations": [{"type": "single", "gate": "Q", "target": 0, "params": []}]}',
     "Unknown gate: Q"),
    ('{"num_qubits": 1, "num_classical_bits": 1, "operations": [{"type": "channel", "channel": "Bit", "target": 0, "params": []}]}',
     "Unknown noise channel: Bit"),
    ('{"num_qubits": 1, "num_classical_bits": 1, "operations": [{"type": "toffoli"}]}', "unknown variant `toffoli`"),
    ('{"num_qubits": 1.5, "num_classical_bits": 1, "operations": []}', "expected usize"),
])
def test_json_rejections(doc, needle):
    with pytest.raises(qf.QuantumError) as e:
        qf.Circuit.from_json(doc)
    assert needle in str(e.value)


def test_json_missing_angle_reads_zero_and_unknown_fields_are_ignored():
    c = qf.Circuit.from_json('{"num_qubits": 1, "num_classical_bits": 1, "extra": [1, {"a": null}], '
                             '"operations": [{"type": "single", "gate": "Rx", "target": 0, "params": [], "note": "x"}]}')
    assert float(c.ops()[0]["theta"]) == 0.0 and int(c.ops()[0]["gate"]) == A.GATE_RX
