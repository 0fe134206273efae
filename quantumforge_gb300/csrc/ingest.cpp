// ingest.cpp — circuit formats to and from the qf_op array: OpenQASM 2.0
// import (parse_qasm, src/qasm.rs:73-1075), QASM export (export_qasm,
// src/qasm_export.rs), and the JSON form of Circuit (SerializedCircuit,
// src/serialize.rs:9-170, 226-366). Host code only; the statement handling
// follows the reference's parser line for line in behaviour (statement
// splitting, register resolution, the expression evaluator and its `pi` / `e`
// substitution, user gate expansion), so a circuit file yields the same op
// list here as there. Where the reference would panic on malformed input (a
// gate with too few qubit arguments or parameters), this returns an error.
#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <string_view>
#include <vector>

#include "qf_internal.h"

namespace qf {
namespace {

using std::string;
using std::string_view;

string_view trim(string_view s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

bool starts_with(string_view s, string_view p) { return s.size() >= p.size() && s.compare(0, p.size(), p) == 0; }

string_view trim_end_semicolons(string_view s) {
    while (!s.empty() && s.back() == ';') s.remove_suffix(1);
    return s;
}

std::vector<string_view> split(string_view s, char sep) {
    std::vector<string_view> out;
    size_t start = 0;
    for (;;) {
        const size_t p = s.find(sep, start);
        if (p == string_view::npos) {
            out.push_back(s.substr(start));
            return out;
        }
        out.push_back(s.substr(start, p - start));
        start = p + 1;
    }
}

// usize::from_str: optional '+', then one or more ASCII digits.
bool parse_usize(string_view s, uint64_t *out) {
    if (!s.empty() && s[0] == '+') s.remove_prefix(1);
    if (s.empty()) return false;
    uint64_t v = 0;
    for (char c : s) {
        if (c < '0' || c > '9') return false;
        const uint64_t d = (uint64_t)(c - '0');
        if (v > (UINT64_MAX - d) / 10) return false;
        v = v * 10 + d;
    }
    *out = v;
    return true;
}

// f64::from_str on the strings this parser hands it (digits, dots, signs,
// exponents): the whole string must convert.
bool parse_f64(string_view s, double *out) {
    if (s.empty()) return false;
    string t(s);
    char *end = nullptr;
    const double v = std::strtod(t.c_str(), &end);
    if (end != t.c_str() + t.size()) return false;
    for (char c : t)  // strtod also reads inf/nan/hex, which f64::from_str spells differently
        if (!(std::isdigit((unsigned char)c) || c == '.' || c == '-' || c == '+' || c == 'e' || c == 'E')) return false;
    *out = v;
    return true;
}

// ---- expression evaluator (eval_qasm_expr, src/qasm.rs:913-1071) -----------
enum TokKind { T_NUM, T_PLUS, T_MINUS, T_STAR, T_SLASH, T_LP, T_RP };
struct Tok {
    TokKind k;
    double v;
};

bool tokenize(const string &s, std::vector<Tok> &out) {
    size_t i = 0;
    while (i < s.size()) {
        const char c = s[i];
        if (c == ' ' || c == '\t') { ++i; continue; }
        if (c == '+') { out.push_back({T_PLUS, 0}); ++i; continue; }
        if (c == '-') { out.push_back({T_MINUS, 0}); ++i; continue; }
        if (c == '*') { out.push_back({T_STAR, 0}); ++i; continue; }
        if (c == '/') { out.push_back({T_SLASH, 0}); ++i; continue; }
        if (c == '(') { out.push_back({T_LP, 0}); ++i; continue; }
        if (c == ')') { out.push_back({T_RP, 0}); ++i; continue; }
        if (std::isdigit((unsigned char)c) || c == '.') {
            size_t j = i;
            while (j < s.size() && (std::isdigit((unsigned char)s[j]) || s[j] == '.')) ++j;
            double v;
            if (!parse_f64(string_view(s).substr(i, j - i), &v)) return false;
            out.push_back({T_NUM, v});
            i = j;
            continue;
        }
        return false;
    }
    return true;
}

bool parse_expr(const std::vector<Tok> &t, size_t &p, double *out);

bool parse_factor(const std::vector<Tok> &t, size_t &p, double *out) {
    if (p >= t.size()) return false;
    switch (t[p].k) {
    case T_NUM: *out = t[p++].v; return true;
    case T_MINUS: {
        ++p;
        double v;
        if (!parse_factor(t, p, &v)) return false;
        *out = -v;
        return true;
    }
    case T_PLUS: ++p; return parse_factor(t, p, out);
    case T_LP: {
        ++p;
        double v;
        if (!parse_expr(t, p, &v)) return false;
        if (p >= t.size() || t[p].k != T_RP) return false;
        ++p;
        *out = v;
        return true;
    }
    default: return false;
    }
}

bool parse_term(const std::vector<Tok> &t, size_t &p, double *out) {
    double left;
    if (!parse_factor(t, p, &left)) return false;
    while (p < t.size()) {
        if (t[p].k == T_STAR) {
            ++p;
            double r;
            if (!parse_factor(t, p, &r)) return false;
            left *= r;
        } else if (t[p].k == T_SLASH) {
            ++p;
            double r;
            if (!parse_factor(t, p, &r)) return false;
            if (r == 0.0) return false;
            left /= r;
        } else {
            break;
        }
    }
    *out = left;
    return true;
}

bool parse_expr(const std::vector<Tok> &t, size_t &p, double *out) {
    double left;
    if (!parse_term(t, p, &left)) return false;
    while (p < t.size()) {
        if (t[p].k == T_PLUS) {
            ++p;
            double r;
            if (!parse_term(t, p, &r)) return false;
            left += r;
        } else if (t[p].k == T_MINUS) {
            ++p;
            double r;
            if (!parse_term(t, p, &r)) return false;
            left -= r;
        } else {
            break;
        }
    }
    *out = left;
    return true;
}

void replace_all(string &s, const string &from, const string &to) {
    size_t pos = 0;
    while ((pos = s.find(from, pos)) != string::npos) {
        s.replace(pos, from.size(), to);
        pos += to.size();
    }
}

// `pi` and `e` are replaced textually by the Display of PI and E (so an
// exponent such as 1e-3 is read as 1, E, -3, as the reference reads it).
bool eval_qasm_expr(string_view src, double *out) {
    string s(trim(src));
    if (s.empty()) return false;
    replace_all(s, "pi", "3.141592653589793");
    replace_all(s, "e", "2.718281828459045");
    std::vector<Tok> t;
    if (!tokenize(s, t)) return false;
    size_t p = 0;
    double v;
    if (!parse_expr(t, p, &v) || p != t.size()) return false;
    *out = v;
    return true;
}

bool is_gate_delimiter(char c) { return c == '(' || c == ' ' || c == '['; }

bool is_parameterized_gate(string_view n) {
    static const char *names[] = {"rx", "Rx", "ry", "Ry", "rz", "Rz", "u1", "U1", "u2", "U2", "u3", "U3"};
    for (const char *x : names)
        if (n == x) return true;
    return false;
}

qf_op gate_op(int gate, uint32_t q, double theta = 0.0) {
    qf_op o{};
    o.kind = QF_OP_GATE;
    o.gate = (uint8_t)gate;
    o.q0 = q;
    o.theta = theta;
    return o;
}

qf_op two_op(int kind, uint32_t a, uint32_t b) {
    qf_op o{};
    o.kind = (uint8_t)kind;
    o.q0 = a;
    o.q1 = b;
    return o;
}

struct GateDef {
    std::vector<string> params, qargs;
    struct Stmt {
        string name;
        std::vector<string> params, qargs;
    };
    std::vector<Stmt> body;
};

struct QasmError {
    uint64_t line;
    string message;
};

class QasmParser {
  public:
    explicit QasmParser(string_view src) {
        // str::lines: split on '\n', drop one trailing '\r' per line, no final empty line
        size_t start = 0;
        while (start < src.size()) {
            size_t e = src.find('\n', start);
            if (e == string_view::npos) e = src.size();
            string_view l = src.substr(start, e - start);
            if (!l.empty() && l.back() == '\r') l.remove_suffix(1);
            lines_.push_back(l);
            start = e + 1;
        }
    }

    bool parse(std::vector<qf_op> &ops, QasmError &err) {
        bool header_seen = false;
        while (!pending_.empty() || pos_ < lines_.size()) {
            string held;
            string_view raw;
            if (!pending_.empty()) {
                held = pending_.front();
                pending_.pop_front();
                raw = held;
            } else {
                raw = trim(lines_[pos_]);
                ++pos_;
            }
            if (raw.empty() || starts_with(raw, "//")) continue;
            if (starts_with(raw, "/*") && raw.size() >= 2 && raw.substr(raw.size() - 2) == "*/") continue;
            if (starts_with(raw, "OPENQASM")) {
                header_seen = true;
                continue;
            }
            if (starts_with(raw, "include")) continue;
            if (!header_seen) return fail_at(err, "missing OPENQASM 2.0 header");
            string_view line = raw;
            string first;
            if (raw.find('{') == string_view::npos && raw.find('}') == string_view::npos) {
                std::vector<string> segs;
                for (string_view s : split(raw, ';')) {
                    s = trim(s);
                    if (!s.empty()) segs.emplace_back(s);
                }
                for (size_t k = segs.size(); k-- > 1;) pending_.push_front(segs[k]);
                first = segs.empty() ? string() : segs[0];
                line = first;
            }
            if (line.empty() || starts_with(line, "//")) continue;
            bool ok;
            if (starts_with(line, "qreg")) ok = parse_reg(line, "qreg", qregs_, qubit_count_, err);
            else if (starts_with(line, "creg")) ok = parse_reg(line, "creg", cregs_, cbit_count_, err);
            else if (starts_with(line, "gate")) ok = parse_gate_def(line, err);
            else if (starts_with(line, "barrier")) ok = true;  // a no-op in simulation
            else if (starts_with(line, "reset"))
                ok = fail_at(err, "reset is not supported in pure-state simulation (requires measure+conditional-X; use shot "
                                  "execution mode)");
            else if (starts_with(line, "measure")) ok = parse_measure(line, ops, err);
            else ok = parse_gate_application(line, ops, err);
            if (!ok) return false;
        }
        return true;
    }

    uint64_t qubits() const { return qubit_count_; }
    uint64_t cbits() const { return cbit_count_; }

  private:
    std::vector<string_view> lines_;
    std::deque<string> pending_;
    size_t pos_ = 0;
    std::map<string, std::pair<uint64_t, uint64_t>> qregs_, cregs_;
    uint64_t qubit_count_ = 0, cbit_count_ = 0;
    std::map<string, GateDef> defs_;

    bool fail_at(QasmError &err, string msg) {
        err.line = pos_;
        err.message = std::move(msg);
        return false;
    }

    // parse_reg_decl (src/qasm.rs:902-911)
    static bool reg_decl(string_view s, string &name, uint64_t &size) {
        s = trim(s);
        const size_t b0 = s.find('['), b1 = s.find(']');
        if (b0 == string_view::npos || b1 == string_view::npos || b1 < b0) return false;
        name = string(trim(s.substr(0, b0)));
        return parse_usize(trim(s.substr(b0 + 1, b1 - b0 - 1)), &size);
    }

    bool parse_reg(string_view line, const char *kw, std::map<string, std::pair<uint64_t, uint64_t>> &regs, uint64_t &count,
                   QasmError &err) {
        line = trim(trim_end_semicolons(line));
        string name;
        uint64_t size;
        if (!reg_decl(line.substr(std::strlen(kw)), name, size)) return fail_at(err, string("invalid ") + kw + " declaration");
        regs[name] = {count, size};
        count += size;
        return true;
    }

    bool resolve(string_view ref, const std::map<string, std::pair<uint64_t, uint64_t>> &regs, bool quantum, uint64_t &out,
                 QasmError &err) {
        const char *what = quantum ? "qubit" : "classical bit";
        const size_t b0 = ref.find('[');
        if (b0 != string_view::npos) {
            const string name(trim(ref.substr(0, b0)));
            const size_t b1 = ref.find(']');
            if (b1 == string_view::npos || b1 < b0)
                return fail_at(err, string("invalid ") + (quantum ? "qubit" : "classical bit") + " reference '" + string(ref) + "'");
            const string_view idx_s = ref.substr(b0 + 1, b1 - b0 - 1);
            uint64_t idx;
            if (!parse_usize(trim(idx_s), &idx))
                return fail_at(err, string("invalid ") + what + " index '" + string(idx_s) + "'");
            auto it = regs.find(name);
            if (it == regs.end())
                return fail_at(err, string("unknown ") + (quantum ? "qubit" : "classical") + " register '" + name + "'");
            if (idx >= it->second.second)
                return fail_at(err, string(what) + " index " + std::to_string(idx) + " out of range for register '" + name +
                                        "' (size " + std::to_string(it->second.second) + ")");
            out = it->second.first + idx;
            return true;
        }
        auto it = regs.find(string(ref));
        if (it == regs.end())
            return fail_at(err, string("unknown ") + (quantum ? "qubit" : "classical") + " register '" + string(ref) + "'");
        out = it->second.first;  // a whole register names its first element
        return true;
    }

    bool parse_measure(string_view line, std::vector<qf_op> &ops, QasmError &err) {
        line = trim(trim_end_semicolons(line));
        string_view rest = line.substr(7);
        std::vector<string_view> parts;
        size_t start = 0;
        for (;;) {
            const size_t p = rest.find("->", start);
            if (p == string_view::npos) {
                parts.push_back(rest.substr(start));
                break;
            }
            parts.push_back(rest.substr(start, p - start));
            start = p + 2;
        }
        if (parts.size() != 2) return fail_at(err, "measure requires 'q[i] -> c[j]'");
        uint64_t q, c;
        if (!resolve(trim(parts[0]), qregs_, true, q, err) || !resolve(trim(parts[1]), cregs_, false, c, err)) return false;
        qf_op o{};
        o.kind = QF_OP_MEASURE;
        o.q0 = (uint32_t)q;
        o.param = (uint32_t)c;
        ops.push_back(o);
        return true;
    }

    // parse_gate_call (src/qasm.rs:691-719): name and the comma-separated qubit arguments.
    bool gate_call(string_view line, string &name, std::vector<string> &qargs, QasmError &err) {
        line = trim(line);
        size_t ne = 0;
        while (ne < line.size() && !is_gate_delimiter(line[ne])) ++ne;
        name = string(line.substr(0, ne));
        string_view qs;
        if (line.find('(') != string_view::npos) {
            const size_t pe = line.find(')');
            if (pe == string_view::npos) return fail_at(err, "unclosed parenthesis in gate call");
            qs = line.substr(pe + 1);
        } else {
            qs = line.substr(ne);
        }
        qargs.clear();
        for (string_view a : split(qs, ',')) {
            a = trim(trim_end_semicolons(trim(a)));
            if (!a.empty()) qargs.emplace_back(a);
        }
        return true;
    }

    bool need(size_t have, size_t want, const string &name, const char *what, QasmError &err) {
        if (have >= want) return true;
        return fail_at(err, "gate '" + name + "' needs " + std::to_string(want) + " " + what + ", got " + std::to_string(have));
    }

    // apply_builtin_gate_on_qubits (src/qasm.rs:583-689)
    bool builtin(const string &g, const std::vector<uint64_t> &ix, std::vector<qf_op> &ops, QasmError &err) {
        struct One {
            const char *names[3];
            int gate;
        };
        static const One ones[] = {{{"x", "X", nullptr}, QF_GATE_X},      {{"y", "Y", nullptr}, QF_GATE_Y},
                                   {{"z", "Z", nullptr}, QF_GATE_Z},      {{"h", "H", nullptr}, QF_GATE_H},
                                   {{"s", "S", nullptr}, QF_GATE_S},      {{"sdg", "Sdg", nullptr}, QF_GATE_SDG},
                                   {{"t", "T", nullptr}, QF_GATE_T},      {{"tdg", "Tdg", nullptr}, QF_GATE_TDG},
                                   {{"id", "I", "Identity"}, QF_GATE_I}};
        for (const One &o : ones)
            for (const char *nm : o.names)
                if (nm && g == nm) {
                    if (!need(ix.size(), 1, g, "qubits", err)) return false;
                    ops.push_back(gate_op(o.gate, (uint32_t)ix[0]));
                    return true;
                }
        const char *cx[] = {"cx", "CX", "cnot", "CNOT"};
        for (const char *nm : cx)
            if (g == nm) {
                if (!need(ix.size(), 2, g, "qubits", err)) return false;
                ops.push_back(two_op(QF_OP_CNOT, (uint32_t)ix[0], (uint32_t)ix[1]));
                return true;
            }
        if (g == "cz" || g == "CZ" || g == "swap" || g == "SWAP") {
            if (!need(ix.size(), 2, g, "qubits", err)) return false;
            ops.push_back(two_op(g == "cz" || g == "CZ" ? QF_OP_CZ : QF_OP_SWAP, (uint32_t)ix[0], (uint32_t)ix[1]));
            return true;
        }
        if (g == "ccx" || g == "CCX" || g == "toffoli") {  // the reference's 15-op decomposition
            if (!need(ix.size(), 3, g, "qubits", err)) return false;
            const uint32_t a = (uint32_t)ix[0], b = (uint32_t)ix[1], c = (uint32_t)ix[2];
            ops.push_back(gate_op(QF_GATE_H, c));
            ops.push_back(two_op(QF_OP_CNOT, b, c));
            ops.push_back(gate_op(QF_GATE_TDG, c));
            ops.push_back(two_op(QF_OP_CNOT, a, c));
            ops.push_back(gate_op(QF_GATE_T, c));
            ops.push_back(two_op(QF_OP_CNOT, b, c));
            ops.push_back(gate_op(QF_GATE_TDG, c));
            ops.push_back(two_op(QF_OP_CNOT, a, c));
            ops.push_back(gate_op(QF_GATE_T, b));
            ops.push_back(gate_op(QF_GATE_T, c));
            ops.push_back(two_op(QF_OP_CNOT, a, b));
            ops.push_back(gate_op(QF_GATE_H, c));
            ops.push_back(gate_op(QF_GATE_T, a));
            ops.push_back(gate_op(QF_GATE_TDG, b));
            ops.push_back(two_op(QF_OP_CNOT, a, b));
            return true;
        }
        return fail_at(err, "unknown gate '" + g + "'");
    }

    // apply_parameterized_gate (src/qasm.rs:775-812): u1 = Rz, u2/u3 as Rz Ry Rz.
    bool parameterized(const string &g, const std::vector<double> &p, const std::vector<uint64_t> &ix, std::vector<qf_op> &ops,
                       QasmError &err) {
        const bool rx = g == "rx" || g == "Rx", ry = g == "ry" || g == "Ry", rz = g == "rz" || g == "Rz";
        const bool u1 = g == "u1" || g == "U1", u2 = g == "u2" || g == "U2", u3 = g == "u3" || g == "U3";
        if (!(rx || ry || rz || u1 || u2 || u3)) return builtin(g, ix, ops, err);
        if (!need(ix.size(), 1, g, "qubits", err)) return false;
        const uint32_t q = (uint32_t)ix[0];
        if (rx || ry || rz || u1) {
            if (!need(p.size(), 1, g, "parameters", err)) return false;
            ops.push_back(gate_op(rx ? QF_GATE_RX : ry ? QF_GATE_RY : QF_GATE_RZ, q, p[0]));
        } else if (u2) {
            if (!need(p.size(), 2, g, "parameters", err)) return false;
            ops.push_back(gate_op(QF_GATE_RZ, q, p[0]));
            ops.push_back(gate_op(QF_GATE_RY, q, 1.5707963267948966));  // FRAC_PI_2
            ops.push_back(gate_op(QF_GATE_RZ, q, p[1]));
        } else {
            if (!need(p.size(), 3, g, "parameters", err)) return false;
            ops.push_back(gate_op(QF_GATE_RZ, q, p[1]));
            ops.push_back(gate_op(QF_GATE_RY, q, p[0]));
            ops.push_back(gate_op(QF_GATE_RZ, q, p[2]));
        }
        return true;
    }

    bool parse_gate_application(string_view line, std::vector<qf_op> &ops, QasmError &err) {
        line = trim(trim_end_semicolons(line));
        size_t ne = 0;
        while (ne < line.size() && !is_gate_delimiter(line[ne])) ++ne;
        const string name(line.substr(0, ne));
        if (defs_.count(name)) return apply_user_gate(line, name, ops, err);
        string g;
        std::vector<string> qargs;
        std::vector<double> params;
        if (is_parameterized_gate(name)) {  // parse_gate_call_with_params (src/qasm.rs:720-773)
            const size_t p0 = line.find('(');
            if (p0 != string_view::npos) {
                const size_t p1 = line.find(')');
                if (p1 == string_view::npos) return fail_at(err, "unclosed parenthesis in gate call");
                for (string_view p : split(line.substr(p0 + 1, p1 - p0 - 1), ',')) {
                    p = trim(p);
                    if (p.empty()) continue;
                    double v;
                    if (!eval_qasm_expr(p, &v)) return fail_at(err, "invalid parameter '" + string(p) + "'");
                    params.push_back(v);
                }
            }
            const size_t pe = line.find(')');
            string_view qs = pe != string_view::npos ? line.substr(pe + 1) : line.substr(ne);
            for (string_view a : split(qs, ',')) {
                a = trim(trim_end_semicolons(trim(a)));
                if (!a.empty()) qargs.emplace_back(a);
            }
            g = name;
        } else if (!gate_call(line, g, qargs, err)) {
            return false;
        }
        std::vector<uint64_t> ix;
        for (const string &a : qargs) {
            uint64_t q;
            if (!resolve(a, qregs_, true, q, err)) return false;
            ix.push_back(q);
        }
        return is_parameterized_gate(name) ? parameterized(g, params, ix, ops, err) : builtin(g, ix, ops, err);
    }

    // apply_user_gate (src/qasm.rs:523-581): inline expansion; call parameters
    // are plain numbers; body parameters are formal names, numbers or 0.
    bool apply_user_gate(string_view line, const string &name, std::vector<qf_op> &ops, QasmError &err) {
        const GateDef def = defs_.at(name);
        string g;
        std::vector<string> qargs;
        if (!gate_call(line, g, qargs, err)) return false;
        if (qargs.size() != def.qargs.size())
            return fail_at(err, "gate '" + name + "' expects " + std::to_string(def.qargs.size()) + " qargs, got " +
                                    std::to_string(qargs.size()));
        std::map<string, uint64_t> amap;
        for (size_t i = 0; i < def.qargs.size(); ++i) {
            uint64_t q;
            if (!resolve(qargs[i], qregs_, true, q, err)) return false;
            amap[def.qargs[i]] = q;
        }
        std::vector<double> call;
        const size_t p0 = line.find('('), p1 = line.find(')');
        if (p0 != string_view::npos && p1 != string_view::npos && p1 > p0) {
            for (string_view p : split(line.substr(p0 + 1, p1 - p0 - 1), ',')) {
                p = trim(p);
                double v;
                if (!p.empty() && parse_f64(p, &v)) call.push_back(v);
            }
        }
        std::map<string, double> pmap;
        for (size_t i = 0; i < def.params.size() && i < call.size(); ++i) pmap[def.params[i]] = call[i];
        for (const GateDef::Stmt &st : def.body) {
            std::vector<uint64_t> ix;
            for (const string &qa : st.qargs) {
                auto it = amap.find(qa);
                ix.push_back(it == amap.end() ? 0 : it->second);
            }
            std::vector<double> ps;
            for (const string &bp : st.params) {
                auto it = pmap.find(bp);
                double v = 0.0;
                if (it != pmap.end()) v = it->second;
                else if (!parse_f64(bp, &v)) v = 0.0;
                ps.push_back(v);
            }
            const bool ok = is_parameterized_gate(st.name) ? parameterized(st.name, ps, ix, ops, err) : builtin(st.name, ix, ops, err);
            if (!ok) return false;
        }
        return true;
    }

    // parse_gate_def / parse_gate_def_body (src/qasm.rs:281-455)
    bool parse_gate_def(string_view first_line, QasmError &err) {
        string header(trim(first_line));
        std::vector<string> body;
        const size_t brace = header.find('{');
        if (brace != string::npos) {
            const string body_part = header.substr(brace + 1);
            header = header.substr(0, brace);
            if (!trim(body_part).empty()) body.push_back(body_part);
        } else {
            while (pos_ < lines_.size()) {
                const string_view next = trim(lines_[pos_]);
                ++pos_;
                if (next.empty() || starts_with(next, "//")) continue;
                const size_t b = next.find('{');
                if (b != string_view::npos) {
                    header = header + " " + string(next.substr(0, b));
                    const string_view bp = next.substr(b + 1);
                    if (!trim(bp).empty()) body.emplace_back(bp);
                    break;
                }
                header = header + " " + string(next);
            }
        }
        int depth = 0;
        while (pos_ < lines_.size()) {
            const string_view next = trim(lines_[pos_]);
            ++pos_;
            if (next.empty() || starts_with(next, "//")) continue;
            for (char ch : next) {
                if (ch == '{') {
                    ++depth;
                } else if (ch == '}') {
                    if (depth == 0) {
                        const string_view before = next.substr(0, next.find('}'));
                        if (!trim(before).empty()) body.emplace_back(before);
                        return gate_def_body(header, body, err);
                    }
                    --depth;
                }
            }
            body.emplace_back(next);
        }
        return fail_at(err, "unclosed gate definition (missing '}')");
    }

    bool gate_def_body(const string &header_in, const std::vector<string> &body_lines, QasmError &err) {
        string_view header = trim(header_in);
        if (starts_with(header, "gate ")) header = trim(header.substr(5));
        const size_t paren = header.find('(');
        size_t ne = paren != string_view::npos ? paren : (header.find(' ') != string_view::npos ? header.find(' ') : header.size());
        GateDef def;
        const string name(trim(header.substr(0, ne)));
        string_view qsrc;
        if (paren != string_view::npos) {
            const size_t pe = header.find(')');
            if (pe == string_view::npos) return fail_at(err, "unclosed parenthesis in gate definition");
            for (string_view p : split(header.substr(paren + 1, pe - paren - 1), ',')) {
                p = trim(p);
                if (!p.empty()) def.params.emplace_back(p);
            }
            qsrc = header.substr(pe + 1);
        } else {
            qsrc = header.substr(ne);
        }
        string qs(qsrc);
        std::replace(qs.begin(), qs.end(), ',', ' ');
        size_t i = 0;
        while (i < qs.size()) {
            while (i < qs.size() && std::isspace((unsigned char)qs[i])) ++i;
            size_t j = i;
            while (j < qs.size() && !std::isspace((unsigned char)qs[j])) ++j;
            if (j > i) def.qargs.push_back(qs.substr(i, j - i));
            i = j;
        }
        string joined;
        for (size_t k = 0; k < body_lines.size(); ++k) {
            if (k) joined += " ";
            joined += body_lines[k];
        }
        for (string_view stmt : split(joined, ';')) {
            stmt = trim(stmt);
            if (stmt.empty()) continue;
            GateDef::Stmt s;
            size_t e = 0;
            while (e < stmt.size() && !is_gate_delimiter(stmt[e])) ++e;
            s.name = string(stmt.substr(0, e));
            string_view qa;
            const size_t p0 = stmt.find('(');
            if (p0 != string_view::npos) {
                const size_t p1 = stmt.find(')');
                if (p1 == string_view::npos) return fail_at(err, "unclosed parenthesis in gate body");
                for (string_view p : split(stmt.substr(p0 + 1, p1 - p0 - 1), ',')) {
                    p = trim(p);
                    if (!p.empty()) s.params.emplace_back(p);
                }
                qa = stmt.substr(p1 + 1);
            } else {
                qa = stmt.substr(s.name.size());
            }
            for (string_view a : split(qa, ',')) {
                a = trim(a);
                if (!a.empty()) s.qargs.emplace_back(a);
            }
            def.body.push_back(std::move(s));
        }
        defs_[name] = std::move(def);
        return true;
    }
};

// ---- JSON (SerializedCircuit, src/serialize.rs) ---------------------------
struct JVal {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } k = NUL;
    bool b = false;
    double num = 0.0;
    bool integral = false;  // written without fraction or exponent
    uint64_t u = 0;         // value when integral and non-negative
    bool negative = false;
    string s;
    std::vector<JVal> arr;
    std::vector<std::pair<string, JVal>> obj;
    const JVal *get(const char *key) const {
        for (const auto &kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

class JsonReader {
  public:
    JsonReader(string_view s) : s_(s) {}
    bool parse(JVal &out, string &err) {
        ws();
        if (!value(out, err, 0)) return false;
        ws();
        if (p_ != s_.size()) return fail(err, "trailing characters");
        return true;
    }

  private:
    string_view s_;
    size_t p_ = 0;
    bool fail(string &err, const char *m) {
        err = string(m) + " at offset " + std::to_string(p_);
        return false;
    }
    void ws() {
        while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\n' || s_[p_] == '\r')) ++p_;
    }
    bool lit(const char *w) {
        const size_t n = std::strlen(w);
        if (s_.substr(p_, n) == w) {
            p_ += n;
            return true;
        }
        return false;
    }
    static void put_utf8(string &o, uint32_t c) {
        if (c < 0x80) o += (char)c;
        else if (c < 0x800) { o += (char)(0xC0 | (c >> 6)); o += (char)(0x80 | (c & 0x3F)); }
        else if (c < 0x10000) { o += (char)(0xE0 | (c >> 12)); o += (char)(0x80 | ((c >> 6) & 0x3F)); o += (char)(0x80 | (c & 0x3F)); }
        else { o += (char)(0xF0 | (c >> 18)); o += (char)(0x80 | ((c >> 12) & 0x3F)); o += (char)(0x80 | ((c >> 6) & 0x3F)); o += (char)(0x80 | (c & 0x3F)); }
    }
    bool hex4(uint32_t &v) {
        if (p_ + 4 > s_.size()) return false;
        v = 0;
        for (int i = 0; i < 4; ++i) {
            const char c = s_[p_++];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else return false;
        }
        return true;
    }
    bool str(string &o, string &err) {
        ++p_;  // opening quote
        while (p_ < s_.size()) {
            const char c = s_[p_++];
            if (c == '"') return true;
            if ((unsigned char)c < 0x20) return fail(err, "control character in string");
            if (c != '\\') { o += c; continue; }
            if (p_ >= s_.size()) break;
            const char e = s_[p_++];
            switch (e) {
            case '"': o += '"'; break;
            case '\\': o += '\\'; break;
            case '/': o += '/'; break;
            case 'b': o += '\b'; break;
            case 'f': o += '\f'; break;
            case 'n': o += '\n'; break;
            case 'r': o += '\r'; break;
            case 't': o += '\t'; break;
            case 'u': {
                uint32_t v;
                if (!hex4(v)) return fail(err, "invalid unicode escape");
                if (v >= 0xD800 && v < 0xDC00) {
                    uint32_t w;
                    if (!(lit("\\u") && hex4(w)) || w < 0xDC00 || w >= 0xE000) return fail(err, "invalid surrogate pair");
                    v = 0x10000 + ((v - 0xD800) << 10) + (w - 0xDC00);
                } else if (v >= 0xDC00 && v < 0xE000) {
                    return fail(err, "invalid surrogate pair");
                }
                put_utf8(o, v);
                break;
            }
            default: return fail(err, "invalid escape");
            }
        }
        return fail(err, "EOF while parsing a string");
    }
    bool number(JVal &v, string &err) {
        const size_t start = p_;
        bool neg = false, frac = false;
        if (s_[p_] == '-') { neg = true; ++p_; }
        if (p_ >= s_.size() || !std::isdigit((unsigned char)s_[p_])) return fail(err, "invalid number");
        if (s_[p_] == '0') ++p_;
        else while (p_ < s_.size() && std::isdigit((unsigned char)s_[p_])) ++p_;
        if (p_ < s_.size() && s_[p_] == '.') {
            frac = true;
            ++p_;
            if (p_ >= s_.size() || !std::isdigit((unsigned char)s_[p_])) return fail(err, "invalid number");
            while (p_ < s_.size() && std::isdigit((unsigned char)s_[p_])) ++p_;
        }
        if (p_ < s_.size() && (s_[p_] == 'e' || s_[p_] == 'E')) {
            frac = true;
            ++p_;
            if (p_ < s_.size() && (s_[p_] == '+' || s_[p_] == '-')) ++p_;
            if (p_ >= s_.size() || !std::isdigit((unsigned char)s_[p_])) return fail(err, "invalid number");
            while (p_ < s_.size() && std::isdigit((unsigned char)s_[p_])) ++p_;
        }
        const string text(s_.substr(start, p_ - start));
        v.k = JVal::NUM;
        v.num = std::strtod(text.c_str(), nullptr);
        v.integral = !frac;
        v.negative = neg;
        if (!frac && !neg) v.integral = parse_usize(text, &v.u);
        return true;
    }
    bool value(JVal &v, string &err, int depth) {
        if (depth > 128) return fail(err, "recursion limit exceeded");
        if (p_ >= s_.size()) return fail(err, "EOF while parsing a value");
        const char c = s_[p_];
        if (c == '{') {
            ++p_;
            v.k = JVal::OBJ;
            ws();
            if (p_ < s_.size() && s_[p_] == '}') { ++p_; return true; }
            for (;;) {
                ws();
                if (p_ >= s_.size() || s_[p_] != '"') return fail(err, "key must be a string");
                string key;
                if (!str(key, err)) return false;
                ws();
                if (p_ >= s_.size() || s_[p_] != ':') return fail(err, "expected ':'");
                ++p_;
                ws();
                JVal x;
                if (!value(x, err, depth + 1)) return false;
                v.obj.emplace_back(std::move(key), std::move(x));
                ws();
                if (p_ < s_.size() && s_[p_] == ',') { ++p_; continue; }
                if (p_ < s_.size() && s_[p_] == '}') { ++p_; return true; }
                return fail(err, "expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p_;
            v.k = JVal::ARR;
            ws();
            if (p_ < s_.size() && s_[p_] == ']') { ++p_; return true; }
            for (;;) {
                ws();
                JVal x;
                if (!value(x, err, depth + 1)) return false;
                v.arr.push_back(std::move(x));
                ws();
                if (p_ < s_.size() && s_[p_] == ',') { ++p_; continue; }
                if (p_ < s_.size() && s_[p_] == ']') { ++p_; return true; }
                return fail(err, "expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.k = JVal::STR;
            return str(v.s, err);
        }
        if (lit("true")) { v.k = JVal::BOOL; v.b = true; return true; }
        if (lit("false")) { v.k = JVal::BOOL; v.b = false; return true; }
        if (lit("null")) { v.k = JVal::NUL; return true; }
        if (c == '-' || std::isdigit((unsigned char)c)) return number(v, err);
        return fail(err, "expected value");
    }
};

bool j_usize(const JVal &o, const char *key, uint64_t &out, string &err) {
    const JVal *v = o.get(key);
    if (!v) { err = string("missing field `") + key + "`"; return false; }
    if (v->k != JVal::NUM || !v->integral || v->negative) { err = string("invalid type for `") + key + "`: expected usize"; return false; }
    out = v->u;
    return true;
}

bool j_str(const JVal &o, const char *key, string &out, string &err) {
    const JVal *v = o.get(key);
    if (!v) { err = string("missing field `") + key + "`"; return false; }
    if (v->k != JVal::STR) { err = string("invalid type for `") + key + "`: expected a string"; return false; }
    out = v->s;
    return true;
}

bool j_f64s(const JVal &o, const char *key, std::vector<double> &out, string &err) {
    const JVal *v = o.get(key);
    if (!v) { err = string("missing field `") + key + "`"; return false; }
    if (v->k != JVal::ARR) { err = string("invalid type for `") + key + "`: expected a sequence"; return false; }
    for (const JVal &x : v->arr) {
        if (x.k != JVal::NUM) { err = string("invalid type in `") + key + "`: expected f64"; return false; }
        out.push_back(x.num);
    }
    return true;
}

const char *kGateNames[] = {"I", "X", "Y", "Z", "H", "S", "Sdg", "T", "Tdg", "Rx", "Ry", "Rz"};
const char *kChannelNames[] = {"Depolarizing", "AmplitudeDamping", "PhaseDamping", "ThermalDamping"};

// deserialize_gate / deserialize_channel (src/serialize.rs:316-366): a missing
// angle or rate reads as 0.
bool j_gate(const string &name, const std::vector<double> &p, int &gate, double &theta, string &err) {
    for (int g = 0; g < 12; ++g)
        if (name == kGateNames[g]) {
            gate = g;
            theta = g >= QF_GATE_RX ? (p.empty() ? 0.0 : p[0]) : 0.0;
            return true;
        }
    err = "Unknown gate: " + name;
    return false;
}

bool ops_from_json(string_view text, std::vector<qf_op> &ops, uint64_t &nq, uint64_t &nc, string &err) {
    JVal root;
    if (!JsonReader(text).parse(root, err)) return false;
    if (root.k != JVal::OBJ) { err = "invalid type: expected struct SerializedCircuit"; return false; }
    if (!j_usize(root, "num_qubits", nq, err) || !j_usize(root, "num_classical_bits", nc, err)) return false;
    const JVal *list = root.get("operations");
    if (!list) { err = "missing field `operations`"; return false; }
    if (list->k != JVal::ARR) { err = "invalid type for `operations`: expected a sequence"; return false; }
    for (const JVal &o : list->arr) {
        if (o.k != JVal::OBJ) { err = "invalid type: expected an operation object"; return false; }
        string type;
        if (!j_str(o, "type", type, err)) return false;
        qf_op op{};
        uint64_t a = 0, b = 0;
        if (type == "single" || type == "conditional") {
            string gname;
            std::vector<double> p;
            if (type == "conditional") {
                uint64_t value;
                if (!j_usize(o, "classical_bit", a, err) || !j_usize(o, "value", value, err)) return false;
                if (value > 255) { err = "invalid value for `value`: expected u8"; return false; }
                if (value > 1) { err = "conditional value must be 0 or 1 (a classical bit holds 0 or 1)"; return false; }
                op.kind = QF_OP_COND;
                op.param = (uint32_t)a;
                op.flags = (uint16_t)value;
            } else {
                op.kind = QF_OP_GATE;
            }
            if (!j_str(o, "gate", gname, err) || !j_usize(o, "target", b, err) || !j_f64s(o, "params", p, err)) return false;
            int g;
            double th;
            if (!j_gate(gname, p, g, th, err)) return false;
            op.gate = (uint8_t)g;
            op.theta = th;
            op.q0 = (uint32_t)b;
        } else if (type == "cx") {
            if (!j_usize(o, "control", a, err) || !j_usize(o, "target", b, err)) return false;
            op = two_op(QF_OP_CNOT, (uint32_t)a, (uint32_t)b);
        } else if (type == "cz" || type == "swap") {
            if (!j_usize(o, "first", a, err) || !j_usize(o, "second", b, err)) return false;
            op = two_op(type == "cz" ? QF_OP_CZ : QF_OP_SWAP, (uint32_t)a, (uint32_t)b);
        } else if (type == "measure") {
            if (!j_usize(o, "target", a, err) || !j_usize(o, "classical_bit", b, err)) return false;
            op.kind = QF_OP_MEASURE;
            op.q0 = (uint32_t)a;
            op.param = (uint32_t)b;
        } else if (type == "channel") {
            string cname;
            std::vector<double> p;
            if (!j_str(o, "channel", cname, err) || !j_usize(o, "target", a, err) || !j_f64s(o, "params", p, err)) return false;
            int kind = -1;
            for (int k = 0; k < 4; ++k)
                if (cname == kChannelNames[k]) kind = k;
            if (kind < 0) { err = "Unknown noise channel: " + cname; return false; }
            op.kind = QF_OP_CHANNEL;
            op.gate = (uint8_t)kind;
            op.q0 = (uint32_t)a;
            op.theta = p.empty() ? 0.0 : p[0];
            if (kind == QF_CHANNEL_THERMAL_DAMPING) qf_op_set_aux(&op, p.size() > 1 ? p[1] : 0.0);
        } else {
            err = "unknown variant `" + type + "`, expected one of `single`, `cx`, `cz`, `swap`, `measure`, `conditional`, `channel`";
            return false;
        }
        if (a > UINT32_MAX || b > UINT32_MAX) { err = "index exceeds the 32-bit range of qf_op"; return false; }
        ops.push_back(op);
    }
    return true;
}

// f64 the way serde_json writes it (the ryu crate's shortest form): integers
// as "1.0", fixed notation for decimal exponents -5 < k <= 16, else d.ddde-7.
string format_f64(double v) {
    if (v == 0.0) return std::signbit(v) ? "-0.0" : "0.0";
    if (!std::isfinite(v)) return "null";
    char buf[64];
    auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::scientific);
    string sci(buf, r.ptr);
    string sign;
    if (sci[0] == '-') {
        sign = "-";
        sci.erase(0, 1);
    }
    const size_t epos = sci.find('e');
    string digits = sci.substr(0, epos);
    const int exp10 = std::stoi(sci.substr(epos + 1));
    digits.erase(std::remove(digits.begin(), digits.end(), '.'), digits.end());
    const int len = (int)digits.size();
    const int kk = exp10 + 1;  // position of the decimal point after the first digit
    string out;
    if (len <= kk && kk <= 16) {
        out = digits + string((size_t)(kk - len), '0') + ".0";
    } else if (0 < kk && kk <= 16) {
        out = digits.substr(0, (size_t)kk) + "." + digits.substr((size_t)kk);
    } else if (-5 < kk && kk <= 0) {
        out = "0." + string((size_t)(-kk), '0') + digits;
    } else if (len == 1) {
        out = digits + "e" + std::to_string(kk - 1);
    } else {
        out = digits.substr(0, 1) + "." + digits.substr(1) + "e" + std::to_string(kk - 1);
    }
    return sign + out;
}

string json_string(const string &s) {
    string o = "\"";
    for (char c : s) {
        switch (c) {
        case '"': o += "\\\""; break;
        case '\\': o += "\\\\"; break;
        case '\n': o += "\\n"; break;
        case '\r': o += "\\r"; break;
        case '\t': o += "\\t"; break;
        default: o += c;
        }
    }
    return o + "\"";
}

// Circuit::to_json (src/serialize.rs:91-163): serde_json's pretty printer,
// two-space indentation, fields in declaration order.
bool ops_to_json(const qf_op *ops, uint64_t n, string &out, string &err) {
    uint64_t mq = 0, mc = 0;
    for (uint64_t k = 0; k < n; ++k) {
        const qf_op &o = ops[k];
        switch (o.kind) {
        case QF_OP_GATE: case QF_OP_CHANNEL: mq = std::max<uint64_t>(mq, o.q0); break;
        case QF_OP_CNOT: case QF_OP_CZ: case QF_OP_SWAP: mq = std::max<uint64_t>(mq, std::max(o.q0, o.q1)); break;
        case QF_OP_MEASURE: case QF_OP_COND:
            mq = std::max<uint64_t>(mq, o.q0);
            mc = std::max<uint64_t>(mc, o.param);
            break;
        default: err = "operation kind " + std::to_string(o.kind) + " is not a Circuit operation"; return false;
        }
    }
    auto params = [](const std::vector<double> &p, const string &ind) {
        if (p.empty()) return string("[]");
        string s = "[\n";
        for (size_t i = 0; i < p.size(); ++i) s += ind + "  " + format_f64(p[i]) + (i + 1 < p.size() ? ",\n" : "\n");
        return s + ind + "]";
    };
    out = "{\n  \"num_qubits\": " + std::to_string(mq + 1) + ",\n  \"num_classical_bits\": " + std::to_string(mc + 1) +
          ",\n  \"operations\": ";
    if (n == 0) {
        out += "[]\n}";
        return true;
    }
    out += "[\n";
    const string I = "      ";
    for (uint64_t k = 0; k < n; ++k) {
        const qf_op &o = ops[k];
        std::vector<std::pair<string, string>> f;
        auto gate = [&](std::vector<std::pair<string, string>> &ff) {
            if (o.gate > QF_GATE_RZ) return false;
            ff.push_back({"gate", json_string(kGateNames[o.gate])});
            ff.push_back({"target", std::to_string(o.q0)});
            std::vector<double> p;
            if (o.gate >= QF_GATE_RX) p.push_back(o.theta);
            ff.push_back({"params", params(p, I)});
            return true;
        };
        switch (o.kind) {
        case QF_OP_GATE:
            f.push_back({"type", "\"single\""});
            if (!gate(f)) { err = "unknown gate code"; return false; }
            break;
        case QF_OP_CNOT: f = {{"type", "\"cx\""}, {"control", std::to_string(o.q0)}, {"target", std::to_string(o.q1)}}; break;
        case QF_OP_CZ: f = {{"type", "\"cz\""}, {"first", std::to_string(o.q0)}, {"second", std::to_string(o.q1)}}; break;
        case QF_OP_SWAP: f = {{"type", "\"swap\""}, {"first", std::to_string(o.q0)}, {"second", std::to_string(o.q1)}}; break;
        case QF_OP_MEASURE:
            f = {{"type", "\"measure\""}, {"target", std::to_string(o.q0)}, {"classical_bit", std::to_string(o.param)}};
            break;
        case QF_OP_COND:
            f = {{"type", "\"conditional\""}, {"classical_bit", std::to_string(o.param)}, {"value", std::to_string(o.flags & 1)}};
            if (!gate(f)) { err = "unknown gate code"; return false; }
            break;
        case QF_OP_CHANNEL: {
            if (o.gate > QF_CHANNEL_THERMAL_DAMPING) { err = "unknown channel code"; return false; }
            std::vector<double> p{o.theta};
            if (o.gate == QF_CHANNEL_THERMAL_DAMPING) p.push_back(qf_op_aux(&o));
            f = {{"type", "\"channel\""}, {"channel", json_string(kChannelNames[o.gate])}, {"target", std::to_string(o.q0)},
                 {"params", params(p, I)}};
            break;
        }
        }
        out += "    {\n";
        for (size_t i = 0; i < f.size(); ++i) out += I + "\"" + f[i].first + "\": " + f[i].second + (i + 1 < f.size() ? ",\n" : "\n");
        out += string("    }") + (k + 1 < n ? ",\n" : "\n");
    }
    out += "  ]\n}";
    return true;
}

// format_angle (src/qasm_export.rs): multiples 1/k of pi by name, else ten
// decimals with trailing zeros dropped.
string format_angle(double angle) {
    const double pi = 3.141592653589793;
    if (std::fabs(angle) < 1e-12) return "0";
    const double ratio = angle / pi;
    if (std::fabs(ratio) > 1e-10) {
        const double r = std::round(1.0 / ratio);
        const int64_t denom = r >= 9.2e18 ? INT64_MAX : (r <= -9.2e18 ? INT64_MIN : (int64_t)r);
        if (denom != 0 && std::fabs(ratio - 1.0 / (double)denom) < 1e-10) {
            if (denom == 1) return "pi";
            if (denom == -1) return "-pi";
            if (denom > 0) return "pi/" + std::to_string(denom);
            return "-pi/" + std::to_string(-denom);
        }
    }
    char buf[512];
    std::snprintf(buf, sizeof buf, "%.10f", angle);
    string s(buf);
    while (!s.empty() && s.back() == '0') s.pop_back();
    while (!s.empty() && s.back() == '.') s.pop_back();
    return s;
}

// export_qasm / export_qasm_with_qubits (src/qasm_export.rs): channels are
// dropped, SWAP becomes three CX, a conditional needs a measured register.
bool ops_to_qasm(const qf_op *ops, uint64_t n, int64_t want_qubits, string &out, string &err) {
    uint64_t mq = 0, mc = 0;
    bool meas = false;
    for (uint64_t k = 0; k < n; ++k) {
        const qf_op &o = ops[k];
        switch (o.kind) {
        case QF_OP_GATE: case QF_OP_CHANNEL: mq = std::max<uint64_t>(mq, o.q0); break;
        case QF_OP_CNOT: case QF_OP_CZ: case QF_OP_SWAP: mq = std::max<uint64_t>(mq, std::max(o.q0, o.q1)); break;
        case QF_OP_MEASURE: meas = true; /* fallthrough */
        case QF_OP_COND:
            mq = std::max<uint64_t>(mq, o.q0);
            mc = std::max<uint64_t>(mc, o.param);
            break;
        default: err = "operation kind " + std::to_string(o.kind) + " is not a Circuit operation"; return false;
        }
    }
    uint64_t nq = n == 0 ? 0 : mq + 1;
    if (want_qubits >= 0) {
        if (nq > (uint64_t)want_qubits) { err = "circuit uses a qubit outside the declared register"; return false; }
        nq = (uint64_t)want_qubits;
    }
    const uint64_t nc = mc + 1;
    static const char *qn[] = {"id", "x", "y", "z", "h", "s", "sdg", "t", "tdg", "rx", "ry", "rz"};
    auto gname = [&](const qf_op &o) {
        string g = qn[o.gate];
        if (o.gate >= QF_GATE_RX) g += "(" + format_angle(o.theta) + ")";
        return g;
    };
    auto q = [](uint32_t i) { return "q[" + std::to_string(i) + "]"; };
    std::vector<string> lines = {"OPENQASM 2.0;", "include \"qelib1.inc\";", ""};
    if (nq > 0) lines.push_back("qreg q[" + std::to_string(nq) + "];");
    if (meas) lines.push_back("creg c[" + std::to_string(nc) + "];");
    lines.push_back("");
    for (uint64_t k = 0; k < n; ++k) {
        const qf_op &o = ops[k];
        if ((o.kind == QF_OP_GATE || o.kind == QF_OP_COND) && o.gate > QF_GATE_RZ) { err = "unknown gate code"; return false; }
        switch (o.kind) {
        case QF_OP_GATE: lines.push_back(gname(o) + " " + q(o.q0) + ";"); break;
        case QF_OP_CNOT: lines.push_back("cx " + q(o.q0) + ", " + q(o.q1) + ";"); break;
        case QF_OP_CZ: lines.push_back("cz " + q(o.q0) + ", " + q(o.q1) + ";"); break;
        case QF_OP_SWAP:
            lines.push_back("cx " + q(o.q0) + ", " + q(o.q1) + ";\ncx " + q(o.q1) + ", " + q(o.q0) + ";\ncx " + q(o.q0) + ", " +
                            q(o.q1) + ";");
            break;
        case QF_OP_MEASURE: lines.push_back("measure " + q(o.q0) + " -> c[" + std::to_string(o.param) + "];"); break;
        case QF_OP_COND:
            if (meas)
                lines.push_back("if (c[" + std::to_string(o.param) + "] == " + std::to_string(o.flags & 1) + ") " + gname(o) + " " +
                                q(o.q0) + ";");
            break;
        default: break;  // channels have no QASM form
        }
    }
    out.clear();
    for (size_t i = 0; i < lines.size(); ++i) {
        if (i) out += "\n";
        out += lines[i];
    }
    return true;
}

int copy_ops(const std::vector<qf_op> &v, qf_op *out, uint64_t capacity, uint64_t *n_out) {
    if (n_out) *n_out = v.size();
    if (!out) return QF_OK;
    if (capacity < v.size())
        return fail(QF_ERR_INVALID_ARGUMENT, "the op buffer holds %llu records, %llu needed", (unsigned long long)capacity,
                    (unsigned long long)v.size());
    if (!v.empty()) std::memcpy(out, v.data(), sizeof(qf_op) * v.size());
    return QF_OK;
}

int copy_text(const string &s, char *out, uint64_t capacity, uint64_t *len) {
    if (len) *len = s.size();
    if (!out) return QF_OK;
    if (capacity < s.size() + 1)
        return fail(QF_ERR_INVALID_ARGUMENT, "the text buffer holds %llu bytes, %llu needed", (unsigned long long)capacity,
                    (unsigned long long)(s.size() + 1));
    std::memcpy(out, s.data(), s.size());
    out[s.size()] = '\0';
    return QF_OK;
}

}  // namespace
}  // namespace qf

using namespace qf;

extern "C" {

int qf_parse_qasm(const char *source, uint64_t len, qf_op *ops_out, uint64_t capacity, uint64_t *n_ops, uint32_t *qubits,
                  uint32_t *classical_bits, uint64_t *error_line) {
    clear_error();
    if (!source && len) return fail(QF_ERR_INVALID_ARGUMENT, "source is NULL");
    QasmParser p(string_view(source ? source : "", len));
    std::vector<qf_op> ops;
    QasmError e{0, ""};
    if (error_line) *error_line = 0;
    if (!p.parse(ops, e)) {
        if (error_line) *error_line = e.line;
        return fail(QF_ERR_INVALID_ARGUMENT, "QASM error at line %llu: %s", (unsigned long long)e.line, e.message.c_str());
    }
    if (p.qubits() > UINT32_MAX || p.cbits() > UINT32_MAX) return fail(QF_ERR_INVALID_ARGUMENT, "register sizes exceed 32 bits");
    if (qubits) *qubits = (uint32_t)p.qubits();
    if (classical_bits) *classical_bits = (uint32_t)p.cbits();
    return copy_ops(ops, ops_out, capacity, n_ops);
}

int qf_circuit_from_json(const char *json, uint64_t len, qf_op *ops_out, uint64_t capacity, uint64_t *n_ops, uint32_t *qubits,
                         uint32_t *classical_bits) {
    clear_error();
    if (!json && len) return fail(QF_ERR_INVALID_ARGUMENT, "json is NULL");
    std::vector<qf_op> ops;
    uint64_t nq = 0, nc = 0;
    string err;
    if (!ops_from_json(string_view(json ? json : "", len), ops, nq, nc, err))
        return fail(QF_ERR_INVALID_ARGUMENT, "JSON error: %s", err.c_str());
    if (qubits) *qubits = (uint32_t)std::min<uint64_t>(nq, UINT32_MAX);
    if (classical_bits) *classical_bits = (uint32_t)std::min<uint64_t>(nc, UINT32_MAX);
    return copy_ops(ops, ops_out, capacity, n_ops);
}

int qf_circuit_to_json(const qf_op *ops, uint64_t n_ops, char *out, uint64_t capacity, uint64_t *len) {
    clear_error();
    if (n_ops && !ops) return fail(QF_ERR_INVALID_ARGUMENT, "ops is NULL");
    string s, err;
    if (!ops_to_json(ops, n_ops, s, err)) return fail(QF_ERR_INVALID_ARGUMENT, "%s", err.c_str());
    return copy_text(s, out, capacity, len);
}

int qf_circuit_to_qasm(const qf_op *ops, uint64_t n_ops, int64_t qubits, char *out, uint64_t capacity, uint64_t *len) {
    clear_error();
    if (n_ops && !ops) return fail(QF_ERR_INVALID_ARGUMENT, "ops is NULL");
    string s, err;
    if (!ops_to_qasm(ops, n_ops, qubits, s, err)) return fail(QF_ERR_INVALID_ARGUMENT, "%s", err.c_str());
    return copy_text(s, out, capacity, len);
}

}  // extern "C"
