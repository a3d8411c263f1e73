// qsg_expr.cu -- initial states and potentials given as expressions in the
// language of the reference's calculator (src/Cal.cpp; the FunctorWrapper /
// Functor2DWrapper / Calculator API of include/QuSim.h:502-538), sampled on
// the device.
//
// The language: complex double values; numbers, the variables x (and y in 2D),
// Pi and I, parentheses, unary + and -, ^ (power, right operand a unary
// expression), * /, + -, comparisons < <= > >= == (on real parts; == compares
// the complex values), && and || (1 or 0), c ? a : b, and the functions sin cos
// tan asin acos atan sinh tanh atanh exp log sqrt abs sign and
// gauss(x, mu, sigma) = exp(-((x - mu)/sigma)^2 / 2) / (sqrt(2 pi) sigma).
// Operator precedence and associativity follow src/Cal.cpp:134-418; every
// operand is evaluated (no short circuit), as there.  Two deliberate
// differences, both where the reference's parser cannot accept the input: it
// advances one character past "==" and so fails on it, and it lists sign but
// never parses sign's argument; here both parse.
//
// An expression compiles on the host to a stack program (opcodes and
// constants, at most kMaxCode / kMaxConst) that the host evaluator
// (qsg_expr_eval) and the sampling kernel run the same way.
#include <cuda_runtime.h>
#include <cuda/std/complex>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/qsg.h"
#include "qsg_launch.h"

namespace qsg {
namespace expr {

enum Op : int32_t {
    OP_END = 0,
    OP_CONST,  // + constant index
    OP_VAR,    // + variable slot (0: x, 1: y, 2.. user variables on the host)
    OP_QUEST, OP_OROR, OP_ANDAND,
    OP_GT, OP_LT, OP_GE, OP_LE, OP_EQ,
    OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_POW,
    OP_SIN, OP_COS, OP_TAN, OP_ASIN, OP_ACOS, OP_ATAN,
    OP_SINH, OP_TANH, OP_ATANH, OP_EXP, OP_LOG, OP_SQRT, OP_ABS, OP_SIGN,
    OP_GAUSS,
};

constexpr int kMaxCode = 512;
constexpr int kMaxConst = 96;
constexpr int kMaxDepth = 32;

struct Program {
    int32_t ncode, nconst, depth, pad;
    int32_t code[kMaxCode];
    double2 consts[kMaxConst];
};

// --- parser -----------------------------------------------------------------

struct Node {
    Op op;
    double2 c{0, 0};
    int var = 0;
    std::vector<std::unique_ptr<Node>> kids;
};
using NodeP = std::unique_ptr<Node>;

struct Parser {
    const char *s;
    const std::map<std::string, int> &vars;  // name -> slot (x, y, user variables)
    std::string err;

    explicit Parser(const char *src, const std::map<std::string, int> &v) : s(src), vars(v) {}

    void skip()
    {
        while (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r') ++s;
    }
    bool take(const char *tok)
    {
        const size_t n = std::strlen(tok);
        if (std::strncmp(s, tok, n) != 0) return false;
        s += n;
        skip();
        return true;
    }
    static bool alpha(char c) { return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || c == '_'; }
    static bool digit(char c) { return c >= '0' && c <= '9'; }

    NodeP mk(Op op, std::vector<NodeP> kids = {})
    {
        NodeP n(new Node());
        n->op = op;
        n->kids = std::move(kids);
        return n;
    }
    NodeP fail(const std::string &m)
    {
        if (err.empty()) err = m;
        return nullptr;
    }

    // question := oror ('?' question ':' oror)*
    NodeP question()
    {
        NodeP a = oror();
        while (a && *s == '?') {
            take("?");
            NodeP b = question();
            if (!b) return nullptr;
            if (!take(":")) return fail(std::string("expected ':' before: ") + s);
            NodeP c = oror();
            if (!c) return nullptr;
            std::vector<NodeP> k;
            k.push_back(std::move(a));
            k.push_back(std::move(b));
            k.push_back(std::move(c));
            a = mk(OP_QUEST, std::move(k));
        }
        return a;
    }
    template <class F> NodeP left_assoc(F next, const std::vector<std::pair<const char *, Op>> &ops)
    {
        NodeP a = (this->*next)();
        for (;;) {
            if (!a) return nullptr;
            bool hit = false;
            for (const auto &o : ops) {
                if (take(o.first)) {
                    NodeP b = (this->*next)();
                    if (!b) return nullptr;
                    std::vector<NodeP> k;
                    k.push_back(std::move(a));
                    k.push_back(std::move(b));
                    a = mk(o.second, std::move(k));
                    hit = true;
                    break;
                }
            }
            if (!hit) return a;
        }
    }
    NodeP oror() { return left_assoc(&Parser::andand, {{"||", OP_OROR}}); }
    NodeP andand() { return left_assoc(&Parser::cmp, {{"&&", OP_ANDAND}}); }
    // two-character comparisons are tried before their one-character prefixes
    NodeP cmp()
    {
        return left_assoc(&Parser::add, {{"<=", OP_LE}, {">=", OP_GE}, {"==", OP_EQ}, {"<", OP_LT}, {">", OP_GT}});
    }
    NodeP add() { return left_assoc(&Parser::mul, {{"+", OP_ADD}, {"-", OP_SUB}}); }
    NodeP mul() { return left_assoc(&Parser::unary, {{"*", OP_MUL}, {"/", OP_DIV}}); }
    // unary := ('-' | '+') pow | pow
    NodeP unary()
    {
        if (take("-")) {
            NodeP a = pow_();
            if (!a) return nullptr;
            std::vector<NodeP> k;
            k.push_back(std::move(a));
            return mk(OP_NEG, std::move(k));
        }
        if (take("+")) return pow_();
        return pow_();
    }
    // pow := atom ('^' unary)?
    NodeP pow_()
    {
        NodeP a = atom();
        if (a && take("^")) {
            NodeP b = unary();
            if (!b) return nullptr;
            std::vector<NodeP> k;
            k.push_back(std::move(a));
            k.push_back(std::move(b));
            a = mk(OP_POW, std::move(k));
        }
        return a;
    }
    NodeP atom()
    {
        if (digit(*s)) {
            char *end = nullptr;
            const double v = std::strtod(s, &end);
            if (end == s) return fail(std::string("failed to parse a number at: ") + s);
            s = end;
            skip();
            NodeP n = mk(OP_CONST);
            n->c = double2{v, 0.0};
            return n;
        }
        if (take("(")) {
            NodeP e = question();
            if (!e) return nullptr;
            if (!take(")")) return fail(std::string("expected ')' before: ") + s);
            return e;
        }
        if (alpha(*s)) {
            std::string name;
            while (alpha(*s) || digit(*s)) name += *s++;
            skip();
            if (*s == '(') {
                static const std::map<std::string, Op> fn1 = {
                    {"sin", OP_SIN},   {"cos", OP_COS},   {"tan", OP_TAN},   {"asin", OP_ASIN}, {"acos", OP_ACOS},
                    {"atan", OP_ATAN}, {"sinh", OP_SINH}, {"tanh", OP_TANH}, {"atanh", OP_ATANH},
                    {"exp", OP_EXP},   {"log", OP_LOG},   {"sqrt", OP_SQRT}, {"abs", OP_ABS},   {"sign", OP_SIGN}};
                take("(");
                std::vector<NodeP> args;
                for (;;) {
                    NodeP a = question();
                    if (!a) return nullptr;
                    args.push_back(std::move(a));
                    if (take(",")) continue;
                    if (take(")")) break;
                    return fail(std::string("expected ',' or ')' before: ") + s);
                }
                if (name == "gauss") {
                    if (args.size() != 3) return fail("gauss takes 3 arguments");
                    return mk(OP_GAUSS, std::move(args));
                }
                auto it = fn1.find(name);
                if (it == fn1.end()) return fail("unknown function: " + name);
                if (args.size() != 1) return fail(name + " takes 1 argument");
                return mk(it->second, std::move(args));
            }
            if (name == "Pi") {
                NodeP n = mk(OP_CONST);
                n->c = double2{3.14159265358979323846, 0.0};
                return n;
            }
            if (name == "I") {
                NodeP n = mk(OP_CONST);
                n->c = double2{0.0, 1.0};
                return n;
            }
            auto it = vars.find(name);
            if (it == vars.end()) return fail("var not defined: " + name);
            NodeP n = mk(OP_VAR);
            n->var = it->second;
            return n;
        }
        if (*s == '\0') return fail("unexpected end of the expression");
        return fail(std::string("unexpected: ") + s);
    }
};

// post-order emission; tracks the stack depth
bool emit(const Node &n, Program &p, int &depth, std::string &err)
{
    for (const auto &k : n.kids)
        if (!emit(*k, p, depth, err)) return false;
    const int need = n.op == OP_CONST || n.op == OP_VAR ? 2 : 1;
    if (p.ncode + need > kMaxCode) {
        err = "expression too long";
        return false;
    }
    p.code[p.ncode++] = n.op;
    if (n.op == OP_CONST) {
        if (p.nconst >= kMaxConst) {
            err = "too many constants in the expression";
            return false;
        }
        p.consts[p.nconst] = n.c;
        p.code[p.ncode++] = p.nconst++;
        ++depth;
    } else if (n.op == OP_VAR) {
        p.code[p.ncode++] = n.var;
        ++depth;
    } else {
        depth -= (int)n.kids.size() - 1;
    }
    if (depth > p.depth) p.depth = depth;
    if (p.depth > kMaxDepth) {
        err = "expression nests too deeply";
        return false;
    }
    return true;
}

int compile(const char *src, const std::map<std::string, int> &vars, Program &p, std::string &err)
{
    std::memset(&p, 0, sizeof(p));
    if (!src) {
        err = "null expression";
        return QSG_ERR_ARG;
    }
    Parser ps(src, vars);
    ps.skip();
    NodeP root = ps.question();
    if (root && *ps.s != '\0') ps.fail(std::string("expected the end of the expression, found: ") + ps.s);
    if (!root || !ps.err.empty()) {
        err = ps.err;
        return QSG_ERR_ARG;
    }
    int depth = 0;
    if (!emit(*root, p, depth, err)) return QSG_ERR_ARG;
    p.code[p.ncode++] = OP_END;
    return QSG_OK;
}

// --- evaluation (host and device) -------------------------------------------

template <class Cx> __host__ __device__ inline Cx cx_of(double2 v) { return Cx(v.x, v.y); }

// One body for both sides: instantiated with std::complex and HostMath on the
// host, with cuda::std::complex and DevMath in the sampling kernel; the check of
// host calls from a host-device function does not apply to the host instance.
#pragma nv_exec_check_disable
template <class Cx, class M>
__host__ __device__ inline Cx run(const Program &p, const Cx *vars)
{
    Cx st[kMaxDepth];
    int sp = -1, k = 0;
    for (;;) {
        const int op = p.code[k++];
        switch (op) {
        case OP_END: return st[0];
        case OP_CONST: st[++sp] = cx_of<Cx>(p.consts[p.code[k++]]); break;
        case OP_VAR: st[++sp] = vars[p.code[k++]]; break;
        case OP_QUEST: sp -= 2; st[sp] = st[sp] != Cx(0) ? st[sp + 1] : st[sp + 2]; break;
        case OP_OROR: --sp; st[sp] = (st[sp] != Cx(0) || st[sp + 1] != Cx(0)) ? Cx(1) : Cx(0); break;
        case OP_ANDAND: --sp; st[sp] = (st[sp] != Cx(0) && st[sp + 1] != Cx(0)) ? Cx(1) : Cx(0); break;
        case OP_GT: --sp; st[sp] = Cx(st[sp].real() > st[sp + 1].real() ? 1 : 0); break;
        case OP_LT: --sp; st[sp] = Cx(st[sp].real() < st[sp + 1].real() ? 1 : 0); break;
        case OP_GE: --sp; st[sp] = Cx(st[sp].real() >= st[sp + 1].real() ? 1 : 0); break;
        case OP_LE: --sp; st[sp] = Cx(st[sp].real() <= st[sp + 1].real() ? 1 : 0); break;
        case OP_EQ: --sp; st[sp] = Cx(st[sp] == st[sp + 1] ? 1 : 0); break;
        case OP_ADD: --sp; st[sp] = st[sp] + st[sp + 1]; break;
        case OP_SUB: --sp; st[sp] = st[sp] - st[sp + 1]; break;
        case OP_MUL: --sp; st[sp] = st[sp] * st[sp + 1]; break;
        case OP_DIV: --sp; st[sp] = st[sp] / st[sp + 1]; break;
        case OP_NEG: st[sp] = -st[sp]; break;
        case OP_POW: --sp; st[sp] = M::pow(st[sp], st[sp + 1]); break;
        case OP_SIN: st[sp] = M::sin(st[sp]); break;
        case OP_COS: st[sp] = M::cos(st[sp]); break;
        case OP_TAN: st[sp] = M::tan(st[sp]); break;
        case OP_ASIN: st[sp] = M::asin(st[sp]); break;
        case OP_ACOS: st[sp] = M::acos(st[sp]); break;
        case OP_ATAN: st[sp] = M::atan(st[sp]); break;
        case OP_SINH: st[sp] = M::sinh(st[sp]); break;
        case OP_TANH: st[sp] = M::tanh(st[sp]); break;
        case OP_ATANH: st[sp] = M::atanh(st[sp]); break;
        case OP_EXP: st[sp] = M::exp(st[sp]); break;
        case OP_LOG: st[sp] = M::log(st[sp]); break;
        case OP_SQRT: st[sp] = M::sqrt(st[sp]); break;
        case OP_ABS: st[sp] = Cx(M::abs(st[sp])); break;
        case OP_SIGN: st[sp] = Cx(st[sp].real() > 0 ? 1 : -1); break;
        case OP_GAUSS: {
            sp -= 2;
            const Cx x = st[sp], mu = st[sp + 1], sigma = st[sp + 2];
            const Cx t = (x - mu) / sigma;
            st[sp] = Cx(1.0) / (M::sqrt(Cx(2 * 3.14159265358979323846)) * sigma) * M::exp(Cx(-0.5) * t * t);
            break;
        }
        default: return Cx(0);
        }
    }
}

struct HostMath {
    using C = std::complex<double>;
    static C pow(C a, C b) { return std::pow(a, b); }
    static C sin(C a) { return std::sin(a); }
    static C cos(C a) { return std::cos(a); }
    static C tan(C a) { return std::tan(a); }
    static C asin(C a) { return std::asin(a); }
    static C acos(C a) { return std::acos(a); }
    static C atan(C a) { return std::atan(a); }
    static C sinh(C a) { return std::sinh(a); }
    static C tanh(C a) { return std::tanh(a); }
    static C atanh(C a) { return std::atanh(a); }
    static C exp(C a) { return std::exp(a); }
    static C log(C a) { return std::log(a); }
    static C sqrt(C a) { return std::sqrt(a); }
    static double abs(C a) { return std::abs(a); }
};

struct DevMath {
    using C = cuda::std::complex<double>;
    static __device__ C pow(C a, C b) { return cuda::std::pow(a, b); }
    static __device__ C sin(C a) { return cuda::std::sin(a); }
    static __device__ C cos(C a) { return cuda::std::cos(a); }
    static __device__ C tan(C a) { return cuda::std::tan(a); }
    static __device__ C asin(C a) { return cuda::std::asin(a); }
    static __device__ C acos(C a) { return cuda::std::acos(a); }
    static __device__ C atan(C a) { return cuda::std::atan(a); }
    static __device__ C sinh(C a) { return cuda::std::sinh(a); }
    static __device__ C tanh(C a) { return cuda::std::tanh(a); }
    static __device__ C atanh(C a) { return cuda::std::atanh(a); }
    static __device__ C exp(C a) { return cuda::std::exp(a); }
    static __device__ C log(C a) { return cuda::std::log(a); }
    static __device__ C sqrt(C a) { return cuda::std::sqrt(a); }
    static __device__ double abs(C a) { return cuda::std::abs(a); }
};

// psi0 and V (its real part, as the reference keeps, src/EvolverImpl1D.cpp:46)
// at x_i = x0 + i dx, y_j = y0 + j dy (src/EvolverImpl.h:95-98,
// src/EvolverImpl2D.cpp:39-98), index j + i ny
__global__ void k_sample_expr(const __grid_constant__ Program pp, const __grid_constant__ Program pv, int nx,
                              int ny, double x0, double y0, double dx, double dy, double2 *psi, double *V)
{
    using C = cuda::std::complex<double>;
    const size_t n = (size_t)nx * ny;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / ny), j = (int)(idx - (size_t)i * ny);
        const C vars[2] = {C(x0 + i * dx, 0.0), C(y0 + j * dy, 0.0)};
        const C p = run<C, DevMath>(pp, vars);
        psi[idx] = make_double2(p.real(), p.imag());
        V[idx] = run<C, DevMath>(pv, vars).real();
    }
}

}  // namespace expr

// Compile the psi0 and V expressions of a grid (variables x, and y in 2D)
// and sample them into psi (nx ny complex128) and V (nx ny real) on st.
// QSG_ERR_ARG with the parse error in err, or QSG_ERR_CUDA.
int sample_expr(int dim, const char *psi_expr, const char *v_expr, int nx, int ny, double x0, double y0, double dx,
                double dy, void *psi, double *V, cudaStream_t st, std::string &err)
{
    std::map<std::string, int> vars = {{"x", 0}};
    if (dim == 2) vars["y"] = 1;
    static thread_local expr::Program pp, pv;  // 3.6 KB each: kept off the stack
    if (int rc = expr::compile(psi_expr, vars, pp, err)) {
        err = "psi expression: " + err;
        return rc;
    }
    if (int rc = expr::compile(v_expr, vars, pv, err)) {
        err = "V expression: " + err;
        return rc;
    }
    const size_t n = (size_t)nx * ny;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 65536);
    expr::k_sample_expr<<<blocks, 256, 0, st>>>(pp, pv, nx, ny, x0, y0, dx, dy, static_cast<double2 *>(psi), V);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("expression sampling: ") + cudaGetErrorString(e);
        return QSG_ERR_CUDA;
    }
    return QSG_OK;
}

}  // namespace qsg

extern "C" int qsg_expr_eval(const char *expr, int nvars, const char *const *names, const double *values,
                             double *out)
{
    if (!expr || !out || nvars < 0 || (nvars > 0 && (!names || !values)))
        return qsg::set_last_error(QSG_ERR_ARG, "qsg_expr_eval: null argument");
    std::map<std::string, int> vars;
    for (int i = 0; i < nvars; ++i) {
        if (!names[i]) return qsg::set_last_error(QSG_ERR_ARG, "qsg_expr_eval: null variable name");
        vars[names[i]] = i;
    }
    qsg::expr::Program p;
    std::string err;
    if (int rc = qsg::expr::compile(expr, vars, p, err)) return qsg::set_last_error(rc, "qsg_expr_eval: " + err);
    std::vector<std::complex<double>> vals(nvars > 0 ? nvars : 1);
    for (int i = 0; i < nvars; ++i) vals[i] = std::complex<double>(values[2 * i], values[2 * i + 1]);
    const std::complex<double> r = qsg::expr::run<std::complex<double>, qsg::expr::HostMath>(p, vals.data());
    out[0] = r.real();
    out[1] = r.imag();
    return QSG_OK;
}
