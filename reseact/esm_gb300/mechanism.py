"""Mechanism front end: an .esm ``reaction_systems`` entry -> flat integer/float tables.

The reference never hand-writes its chemistry: EarthSciAST emits the chemistry RHS at run
time from ``reaction_systems`` (``prototypes/reseact_3d_chem/split_common.jl:530-533``,
mechanism schema as in ``prototypes/g2_depsink/g2_nodep.esm:402-1900``).  This module reads
the same schema and lowers it to the tables the CUDA library and the CPU oracle both consume:

* species: the non-constant species, sorted by name (the reference's cell-major layout sorts
  species by name, ``prototypes/reseact_3d_chem/block_jac.jl:27``);
* reactions: reactant (species, integer stoichiometry) and product (species, coefficient)
  lists; constant species (O2, CH4, H2O in SuperFast) are folded into the rate constant;
* a postfix rate program per reaction, evaluated once per cell per macro step (the rates
  depend only on T, P and parameters, and ``tgrad = 0`` holds inside a macro step,
  ``run_reseact.jl:241``);
* the mass-action RHS term list, the analytic block-Jacobian term list, and the symbolic
  fill pattern of the pivot-free LU of W = I - gamma*h*J (the elimination order of
  ``tools/reactant_handoff/rx_traced_integrator.jl:110-135``, natural species order).

Rate-law convention: plain mass action, v = k * prod(x^nu), so 2 HO2 -> ... has rate
k[HO2]^2 and d[HO2]/dt = -2 k[HO2]^2.  The inline golden tests of ``g2_nodep.esm:9-400``
decide it: with this convention the oracle meets all 49 assertions, while the combinatoric
convention (v divided by prod(nu!)) misses 29 of them (tests/test_oracle_golden.py runs both).
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

# Rate-program opcodes (shared with include/reseact_gb300.h RS_OP_*).
OP_CONST, OP_TEMP, OP_PRES, OP_PARAM = 0, 1, 2, 3
OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_POW, OP_NEG = 10, 11, 12, 13, 14, 15
OP_EXP, OP_LOG, OP_LOG10, OP_SQRT = 20, 21, 22, 23

_BINOPS = {"+": OP_ADD, "-": OP_SUB, "*": OP_MUL, "/": OP_DIV, "^": OP_POW}
_UNOPS = {"exp": OP_EXP, "log": OP_LOG, "log10": OP_LOG10, "sqrt": OP_SQRT, "neg": OP_NEG}

MECH_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mechanisms")


@dataclass
class Reaction:
    rid: str
    reactants: list  # [(species_index, nu:int)]
    products: list  # [(species_index, coef:float)]
    prog_ops: list  # postfix opcodes
    prog_vals: list  # operand per opcode (constant value or parameter index)


@dataclass
class Mechanism:
    name: str
    species: list  # active species names, sorted
    defaults: dict  # species name -> default concentration
    params: list  # parameter names (global scalars referenced by rate programs)
    param_values: list
    reactions: list
    combinatoric: bool = False
    tests: list = field(default_factory=list)

    # ---------------------------------------------------------------- derived tables
    @property
    def ns(self):
        return len(self.species)

    @property
    def nr(self):
        return len(self.reactions)

    def param_index(self, name):
        return self.params.index(name)

    def with_params(self, **overrides):
        m = Mechanism(self.name, list(self.species), dict(self.defaults), list(self.params),
                      list(self.param_values), self.reactions, self.combinatoric, self.tests)
        for k, v in overrides.items():
            m.param_values[m.params.index(k)] = float(v)
        return m

    def with_convention(self, combinatoric):
        m = self.with_params()
        m.combinatoric = bool(combinatoric)
        return m

    def net_stoich(self):
        """Dense net stoichiometry [nr, ns] (products minus reactants)."""
        net = np.zeros((self.nr, self.ns))
        for r, rx in enumerate(self.reactions):
            for s, nu in rx.reactants:
                net[r, s] -= nu
            for s, c in rx.products:
                net[r, s] += c
        return net

    def tables(self):
        """Flat tables in the order the C ABI (rs_mechanism) expects.

        The RHS term list is (reaction, species, net) in species-major order so that each
        species' tendency is accumulated over reactions in increasing reaction index: the
        oracle and the CUDA kernels both follow this list, so their sums associate alike.
        """
        ns, nr = self.ns, self.nr
        net = self.net_stoich()
        # reactant table (CSR over reactions)
        rptr, rsp, rnu = [0], [], []
        for rx in self.reactions:
            for s, nu in rx.reactants:
                rsp.append(s)
                rnu.append(int(nu))
            rptr.append(len(rsp))
        # rate programs (CSR)
        pptr, pops, pvals = [0], [], []
        for rx in self.reactions:
            pops.extend(rx.prog_ops)
            pvals.extend(rx.prog_vals)
            pptr.append(len(pops))
        # RHS terms grouped by species (row), reactions ascending
        rhs_ptr, rhs_r, rhs_c = [0], [], []
        for s in range(ns):
            for r in range(nr):
                if net[r, s] != 0.0:
                    rhs_r.append(r)
                    rhs_c.append(net[r, s])
            rhs_ptr.append(len(rhs_r))
        # reaction partials dv_r/dx_q: one per (reaction, distinct reactant)
        part_r, part_q = [], []
        for r, rx in enumerate(self.reactions):
            for s, _nu in rx.reactants:
                part_r.append(r)
                part_q.append(s)
        # Jacobian pattern: (s, q) with some reaction r having q as reactant and net[r, s] != 0
        jpat = set()
        for p, (r, q) in enumerate(zip(part_r, part_q)):
            for s in range(ns):
                if net[r, s] != 0.0:
                    jpat.add((s, q))
        # W = I - gamma h J pattern = J pattern + diagonal; LU fill by symbolic elimination
        wpat = set(jpat) | {(i, i) for i in range(ns)}
        fill = set(wpat)
        for k in range(ns):
            rows = [i for i in range(k + 1, ns) if (i, k) in fill]
            cols = [j for j in range(k + 1, ns) if (k, j) in fill]
            for i in rows:
                for j in cols:
                    fill.add((i, j))
        lu_entries = sorted(fill)  # row-major
        lu_index = {e: n for n, e in enumerate(lu_entries)}
        diag = [lu_index[(i, i)] for i in range(ns)]
        # Jacobian terms: J[s,q] += net[r,s] * partial[p], entries in row-major LU slot order,
        # partials in reaction order within an entry.
        jac_ptr, jac_slot, jac_part, jac_coef = [0], [], [], []
        jslots = sorted(jpat)
        for (s, q) in jslots:
            for p, (r, qq) in enumerate(zip(part_r, part_q)):
                if qq == q and net[r, s] != 0.0:
                    jac_part.append(p)
                    jac_coef.append(net[r, s])
            jac_slot.append(lu_index[(s, q)])
            jac_ptr.append(len(jac_part))
        # Elimination schedule (Doolittle, pivot-free, natural order):
        # for k: for each i>k with (i,k): L[i,k] = W[i,k]*piv_k ; for j>k with (k,j): W[i,j] -= L*W[k,j]
        elim_ptr, elim_lik, elim_upd = [0], [], []  # per (k,i): slot of (i,k); updates list
        upd_ptr, upd_dst, upd_src = [0], [], []
        for k in range(ns):
            rows = [i for i in range(k + 1, ns) if (i, k) in fill]
            cols = [j for j in range(k + 1, ns) if (k, j) in fill]
            for i in rows:
                elim_lik.append(lu_index[(i, k)])
                for j in cols:
                    upd_dst.append(lu_index[(i, j)])
                    upd_src.append(lu_index[(k, j)])
                upd_ptr.append(len(upd_dst))
            elim_ptr.append(len(elim_lik))
        # lower/upper structure for the triangular solves
        lower_ptr, lower_col, lower_slot = [0], [], []  # forward: column-oriented per k
        for k in range(ns):
            for i in range(k + 1, ns):
                if (i, k) in fill:
                    lower_col.append(i)
                    lower_slot.append(lu_index[(i, k)])
            lower_ptr.append(len(lower_col))
        upper_ptr, upper_col, upper_slot = [0], [], []  # backward: row-oriented per i, j ascending
        for i in range(ns):
            for j in range(i + 1, ns):
                if (i, j) in fill:
                    upper_col.append(j)
                    upper_slot.append(lu_index[(i, j)])
            upper_ptr.append(len(upper_col))
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        return dict(
            ns=ns, nr=nr, n_params=len(self.params), combinatoric=int(self.combinatoric),
            react_ptr=i32(rptr), react_species=i32(rsp), react_nu=i32(rnu),
            prog_ptr=i32(pptr), prog_op=i32(pops), prog_val=f64(pvals),
            params=f64(self.param_values),
            rhs_ptr=i32(rhs_ptr), rhs_reaction=i32(rhs_r), rhs_coef=f64(rhs_c),
            n_partials=len(part_r), part_reaction=i32(part_r), part_species=i32(part_q),
            n_lu=len(lu_entries), lu_row=i32([e[0] for e in lu_entries]),
            lu_col=i32([e[1] for e in lu_entries]), lu_diag=i32(diag),
            n_jac=len(jslots), jac_ptr=i32(jac_ptr), jac_slot=i32(jac_slot),
            jac_part=i32(jac_part), jac_coef=f64(jac_coef),
            elim_ptr=i32(elim_ptr), elim_lik=i32(elim_lik), upd_ptr=i32(upd_ptr),
            upd_dst=i32(upd_dst), upd_src=i32(upd_src),
            lower_ptr=i32(lower_ptr), lower_row=i32(lower_col), lower_slot=i32(lower_slot),
            upper_ptr=i32(upper_ptr), upper_col=i32(upper_col), upper_slot=i32(upper_slot),
        )

    def lu_counts(self, order=None):
        """(LU slots, multipliers, updates, lower entries, upper entries) of the pivot-free
        elimination of W = I - gamma h J in the given species order (natural if None)."""
        t = self.tables()
        if order is None:
            return (int(t["n_lu"]), len(t["elim_lik"]), len(t["upd_dst"]),
                    len(t["lower_slot"]), len(t["upper_slot"]))
        ns = self.ns
        net = self.net_stoich()
        pos = {int(s): k for k, s in enumerate(order)}
        fill = {(k, k) for k in range(ns)}
        for r, rx in enumerate(self.reactions):
            for q, _nu in rx.reactants:
                for s in range(ns):
                    if net[r, s] != 0.0:
                        fill.add((pos[s], pos[q]))
        mults = upds = 0
        for k in range(ns):
            rows = [i for i in range(k + 1, ns) if (i, k) in fill]
            cols = [j for j in range(k + 1, ns) if (k, j) in fill]
            mults += len(rows)
            upds += len(rows) * len(cols)
            for i in rows:
                for j in cols:
                    fill.add((i, j))
        low = sum(1 for (i, j) in fill if i > j)
        return len(fill), mults, upds, low, sum(1 for (i, j) in fill if i < j)

    def flop_counts(self, order=None):
        """FP64 operation counts per cell for one ROS23 attempt (sparse, as executed) with the
        LU eliminated in the given species order (natural, as the reference, if None)."""
        t = self.tables()
        nr, ns = self.nr, self.ns
        n_react = int(t["react_ptr"][-1])
        # rate v_r: product of reactant powers times k (mul per factor, squares add a mul)
        rate = sum(int(nu) for nu in t["react_nu"])  # k * x (*x)
        rhs = rate + 2 * len(t["rhs_reaction"])  # mul + add per term
        part = int(t["n_partials"]) * max(1, n_react // max(1, nr))  # ~products per partial
        jac = part + 2 * len(t["jac_part"])
        n_lu, n_mult, n_upd, n_low, n_up = self.lu_counts(order)
        wbuild = n_lu + ns  # scale + diagonal add
        lu = ns + n_mult + 2 * n_upd  # piv, multipliers, updates
        solve = 2 * n_low + 2 * n_up + ns
        stage = 3 * 3 * ns + 6 * ns  # stage combos k2, unew, b3, utilde
        eest = 8 * ns
        total = 3 * rhs + jac + wbuild + lu + 3 * solve + stage + eest
        dense_lu = ns * ns + math.ceil(2 * ns ** 3 / 3) + 6 * ns * ns + 8 * ns
        return dict(rhs=rhs, jac=jac, lu=lu, solve=solve, total=total,
                    dense_equivalent=3 * rhs + jac + dense_lu)


# --------------------------------------------------------------------------- parsing
def _compile_expr(e, templates, var_index, ops, vals, bindings=None):
    """Postfix-compile an .esm expression; n-ary + and * fold left to right."""
    bindings = bindings or {}
    if isinstance(e, bool):
        raise ValueError("boolean in rate expression")
    if isinstance(e, (int, float)):
        ops.append(OP_CONST)
        vals.append(float(e))
        return
    if isinstance(e, str):
        if e in bindings:
            _compile_expr(bindings[e], templates, var_index, ops, vals)
            return
        kind, idx = var_index(e)
        ops.append(kind)
        vals.append(float(idx))
        return
    op = e["op"]
    if op == "apply_expression_template":
        tpl = templates[e["name"]]
        b = dict(e.get("bindings", {}))
        _compile_expr(tpl["body"], templates, var_index, ops, vals, b)
        return
    args = e.get("args", [])
    if op in _UNOPS:
        if len(args) != 1:
            raise ValueError(f"{op} takes one argument")
        _compile_expr(args[0], templates, var_index, ops, vals, bindings)
        ops.append(_UNOPS[op])
        vals.append(0.0)
        return
    if op == "-" and len(args) == 1:
        _compile_expr(args[0], templates, var_index, ops, vals, bindings)
        ops.append(OP_NEG)
        vals.append(0.0)
        return
    if op == "^" and len(args) == 2 and isinstance(args[1], (int, float)) and \
            float(args[1]) in (2.0, 3.0):
        # small integer powers lower to repeated products (exact on both CPU and GPU)
        n = int(args[1])
        for _ in range(n):
            _compile_expr(args[0], templates, var_index, ops, vals, bindings)
        for _ in range(n - 1):
            ops.append(OP_MUL)
            vals.append(0.0)
        return
    if op in _BINOPS:
        if len(args) < 2:
            raise ValueError(f"{op} needs >= 2 arguments")
        if op in ("-", "/", "^") and len(args) != 2:
            raise ValueError(f"{op} takes two arguments")
        _compile_expr(args[0], templates, var_index, ops, vals, bindings)
        for a in args[1:]:
            _compile_expr(a, templates, var_index, ops, vals, bindings)
            ops.append(_BINOPS[op])
            vals.append(0.0)
        return
    raise ValueError(f"unsupported rate op {op!r}")


def from_reaction_system(name, rs, combinatoric=False):
    """Lower one ``reaction_systems`` entry (g2_nodep.esm schema) to a Mechanism."""
    spec = rs["species"]
    consts = {k: float(v.get("default", 0.0)) for k, v in spec.items() if v.get("constant")}
    active = sorted(k for k, v in spec.items() if not v.get("constant"))
    defaults = {k: float(spec[k].get("default", 0.0)) for k in active}
    params, pvals = [], []
    for k, v in rs.get("parameters", {}).items():
        if k in ("T", "P"):
            continue
        params.append(k)
        pvals.append(float(v.get("default", 0.0)))
    for k in sorted(consts):
        params.append(k)
        pvals.append(consts[k])
    templates = rs.get("expression_templates", {})

    def var_index(v):
        if v == "T":
            return OP_TEMP, 0
        if v == "P":
            return OP_PRES, 0
        if v in params:
            return OP_PARAM, params.index(v)
        raise ValueError(f"unknown rate variable {v!r}")

    reactions = []
    for rx in rs["reactions"]:
        ops, vals = [], []
        _compile_expr(rx["rate"], templates, var_index, ops, vals)
        reac = []
        for sub in rx.get("substrates") or []:
            sname, nu = sub["species"], sub.get("stoichiometry", 1)
            if float(nu) != int(nu):
                raise ValueError("non-integer reactant stoichiometry")
            if sname in consts:  # fold the constant reservoir into k
                for _ in range(int(nu)):
                    ops.append(OP_PARAM)
                    vals.append(float(params.index(sname)))
                    ops.append(OP_MUL)
                    vals.append(0.0)
            else:
                reac.append((active.index(sname), int(nu)))
        prods = []
        for pr in rx.get("products") or []:
            pname, c = pr["species"], float(pr.get("stoichiometry", 1))
            if pname in consts:
                continue
            prods.append((active.index(pname), c))
        reactions.append(Reaction(rx.get("id", f"R{len(reactions) + 1}"), reac, prods, ops, vals))
    return Mechanism(name, active, defaults, params, pvals, reactions, combinatoric,
                     rs.get("tests", []))


def load_esm(path_or_doc, system=None, combinatoric=False):
    """Load a mechanism from an .esm document (path or parsed dict)."""
    doc = path_or_doc
    if not isinstance(doc, dict):
        with open(doc) as fh:
            doc = json.load(fh)
    systems = doc["reaction_systems"]
    if system is None:
        if len(systems) != 1:
            raise ValueError(f"choose one of {sorted(systems)}")
        system = next(iter(systems))
    rs = systems[system]
    if "ref" in rs and "reactions" not in rs:
        raise ValueError(f"reaction system {system} is an external $ref ({rs['ref']})")
    return from_reaction_system(system, rs, combinatoric)


def superfast(combinatoric=False):
    """The SuperFast mechanism shipped with the reference (15 species, 3 constant, 27 reactions)."""
    return load_esm(os.path.join(MECH_DIR, "superfast.esm"), "SuperFast", combinatoric)


# --------------------------------------------------------------------------- synthetic
def synthetic(n_species=30, n_reactions=60, seed=20240503, k_lo=1e-6, k_hi=1e2, c_ref=1e-9):
    """Seeded synthetic mass-action mechanism (uni- and bimolecular), non-explosive.

    Rate constants at 298 K are log-uniform in [k_lo, k_hi] s^-1 (first-order equivalent:
    bimolecular constants are divided by the reference concentration ``c_ref`` so that
    k2*c_ref spans the same range); each gets an Arrhenius temperature factor
    exp(B*(1/T - 1/298)) with B uniform in [-1500, 500] K.  Concentrations are in mol/mol.
    Product coefficients of every reaction sum to at most its reactant count (A -> B,
    A -> 0.5 B + 0.5 C, A + B -> C, A + B -> C + D, 2A -> B ...), so total moles never grow:
    no chain branching, bounded trajectories, stiffness from the 1e8 spread of rates alone.
    """
    rng = np.random.default_rng(seed)
    names = [f"S{i:02d}" for i in range(n_species)]
    reactions = []
    for r in range(n_reactions):
        bimol = rng.random() < 0.5
        a = int(rng.integers(n_species))
        reac = [(a, 1)]
        if bimol:
            b = int(rng.integers(n_species))
            reac = [(a, 2)] if b == a else [(a, 1), (b, 1)]
        n_in = 2 if bimol else 1
        used = {s for s, _ in reac}

        def pick():
            p = int(rng.integers(n_species))
            while p in used:
                p = int(rng.integers(n_species))
            used.add(p)
            return p

        shape = int(rng.integers(3))
        if shape == 0:
            prods = [(pick(), 1.0)]
        elif shape == 1:
            prods = [(pick(), 0.5 * n_in), (pick(), 0.5 * n_in)] if n_in == 1 else \
                [(pick(), 1.0), (pick(), 1.0)]
        else:
            prods = [(pick(), float(n_in))]
        k298 = 10.0 ** rng.uniform(math.log10(k_lo), math.log10(k_hi))
        if bimol:
            k298 /= c_ref
        B = float(rng.uniform(-1500.0, 500.0))
        # k = k298 * exp(B/T - B/298) ; postfix: k298 B T / B/298 - exp *
        ops = [OP_CONST, OP_CONST, OP_TEMP, OP_DIV, OP_CONST, OP_SUB, OP_EXP, OP_MUL]
        vals = [k298, B, 0.0, 0.0, B / 298.0, 0.0, 0.0, 0.0]
        reactions.append(Reaction(f"R{r + 1}", reac, prods, ops, vals))
    defaults = {n: 1e-9 for n in names}
    return Mechanism("Synthetic%dx%d" % (n_species, n_reactions), names, defaults, [], [],
                     reactions, False)
