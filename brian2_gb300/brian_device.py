"""``set_device('b200')``: the Brian2 device plugin of the GB300 step engine.

Import this module (or ``import brian2_gb300`` after ``brian2``) to register the
device; scripts then only change their ``set_device`` call.

How the work is split with Brian's own machinery (the device subclasses
``CPPStandaloneDevice``, ``brian2/devices/cpp_standalone/device.py:168``):

* everything that is not the clock-driven step loop -- array initialisation,
  ``Synapses.connect``, variable setting with expressions and random numbers --
  is generated, compiled and run exactly as by ``cpp_standalone``, so the
  constructed network is the reference's, bit for bit;
* the code objects of the step loop (templates ``stateupdate``, ``threshold``,
  ``reset``, ``synapses``, ``synapses_push_spikes``, ``spikemonitor``,
  ``ratemonitor``, ``statemonitor``) are translated by
  :class:`B200CodeGenerator` and collected into a network *spec*; ``run()``
  records the run instead of queueing ``Network::run`` into ``main``;
* after ``main`` has run, the recorded runs execute on the GPU through the
  ctypes C ABI (:mod:`brian2_gb300.runtime`), and the final state and monitor
  contents are written into the standalone results directory in the
  reference's file format, so ``get_value`` / ``SpikeMonitor.t`` etc. work
  unchanged (``device.py:544-585``).

Limits (raise ``NotImplementedError``, which Brian's test runner treats as
"not supported by this device"): one clock for all step-loop objects (but
``run_regularly`` operations in the start and end slots may run every k-th
step); no host
code between two ``run()`` calls other than assignments of values to neuron-group
state variables (applied between the device runs); random numbers inside the step loop other
than one ``rand()`` per neuron in threshold code (PoissonGroup) and the
binomial draws of ``PoissonInput`` without its normal approximation (both need
``openmp_threads = 0``); synaptic statements that write a neuron variable
other than by ``+=``/``-=``; state monitors outside the ``start`` and ``end``
slots; custom events.
"""
from __future__ import annotations

import json
import os
import re
import time

import numpy as np

from brian2.codegen.generators.cpp_generator import CPPCodeGenerator, c_data_type
from brian2.core.clocks import Clock
from brian2.core.functions import DEFAULT_FUNCTIONS, Function
from brian2.core.preferences import prefs
from brian2.core.variables import ArrayVariable, Constant, DynamicArrayVariable
from brian2.groups.group import CodeRunner
from brian2.devices.cpp_standalone.codeobject import CPPStandaloneCodeObject
from brian2.devices.cpp_standalone.device import CPPStandaloneDevice
from brian2.devices.device import all_devices
from brian2.groups.neurongroup import NeuronGroup
from brian2.groups.subgroup import Subgroup
from brian2.input.binomial import BinomialFunction
from brian2.input.poissongroup import PoissonGroup
from brian2.input.poissoninput import PoissonInput
from brian2.input.spikegeneratorgroup import SpikeGeneratorGroup
from brian2.monitors.ratemonitor import PopulationRateMonitor
from brian2.monitors.spikemonitor import EventMonitor, SpikeMonitor
from brian2.monitors.statemonitor import StateMonitor
from brian2.synapses.synapses import Synapses, SynapticPathway
from brian2.utils.logger import get_logger
from brian2.utils.stringtools import get_identifiers, stripped_deindented_lines

logger = get_logger(__name__)

STEP_TEMPLATES = {"stateupdate", "threshold", "reset", "synapses", "synapses_push_spikes",
                  "spikemonitor", "ratemonitor", "statemonitor", "spikegenerator", "summed_variable"}

# the constants of Brian's C++ binomial sampler by inversion, as it prints them
# (brian2/input/binomial.py:93-141): qn, bound, n, P, Q and the returned count
_NUM = r"([-+0-9.eE]+)"
_BINOM_RE = re.compile(r"double px = " + _NUM + r";.*?if \(X > " + _NUM + r"\).*?"
                       r"px = \(\((\d+)-X\+1\) \* " + _NUM + r" \* px\)/\(X\*" + _NUM + r"\);.*?"
                       r"return ([^;]+);", re.S)


_NORMAL_RE = re.compile(r"return _randn\(vectorisation_idx\) \* " + _NUM + r" \+ " + _NUM + r";")


def draws_random(spec):
    """Whether the step loop of a spec draws from the reference's generator."""
    return bool(spec.get("draws"))


def _draw_calls(code, kind):
    """Rewrites the calls of rand()/randn() in vector code for a draw site (one
    macro per call, in code order); returns (code, number of calls).  Each call
    must run once per neuron: none in a conditional expression."""
    name = {"rand": "_rand(", "randn": "_randn("}[kind]
    lines = code.split("\n")
    for ln in lines:
        if name in ln and ("?" in ln or "&&" in ln or "||" in ln):
            raise NotImplementedError(f"b200: {kind}() in a conditional expression")
    return code, code.count(name)


class B200CodeGenerator(CPPCodeGenerator):
    """C++ generator for device code.

    Produces the same scalar and vector code as ``CPPCodeGenerator`` (the
    vector code is also what the CPU oracle executes) and, for synaptic
    ``on_pre`` code, a device variant in which every in-place update of a
    non-synaptic variable (``ge_post += w``) is an atomic accumulation, since
    many synapses of one step may target the same neuron.
    """

    class_name = "b200_cuda"

    def translate_statement_sequence(self, sc_statements, ve_statements):
        sc_code, ve_code, kwds = super().translate_statement_sequence(sc_statements, ve_statements)
        if self.template_name == "synapses":
            kwds["vector_code_device"] = {name: self._device_block(stmts) for name, stmts in ve_statements.items()}
        return sc_code, ve_code, kwds

    def _device_block(self, statements):
        read, write, indices, cond_write = self.arrays_helper(statements)
        atomic = {v for v in write if self.variable_indices[v] not in ("_idx", "0")}
        for stmt in statements:
            ids = get_identifiers(stmt.expr)
            if ids & atomic:
                raise NotImplementedError(
                    f"b200: on_pre code reads the non-synaptic variable(s) {sorted(ids & atomic)} it updates")
            if stmt.var in atomic:
                if stmt.op not in ("+=", "-=") or (stmt.used_boolean_variables and
                                                   len(stmt.used_boolean_variables)):
                    raise NotImplementedError(
                        f"b200: '{stmt.var} {stmt.op} ...' on a non-synaptic variable; only += and -= "
                        "(atomic accumulation) are supported in synaptic code")
        lines = []
        lines += self.translate_to_read_arrays(read - atomic, write - atomic, indices)
        lines += self.translate_to_declarations(read - atomic, write - atomic, indices)
        for stmt in statements:
            if stmt.var in atomic:
                var = self.variables[stmt.var]
                ptr = self.get_array_name(var)
                idx = self.variable_indices[stmt.var]
                ctype = self.c_data_type(var.dtype)
                expr = self.translate_expression(stmt.expr)
                sign = "" if stmt.op == "+=" else "-"
                line = f"_b200_atomic_add(&{ptr}[{idx}], ({ctype})({sign}({expr})));"
                if stmt.var in cond_write:
                    line = f"if({cond_write[stmt.var]}) {line}"
                lines.append(line)
            else:
                line = self.translate_statement(stmt)
                if stmt.var in cond_write:
                    lines.append(f"if({cond_write[stmt.var]})")
                    lines.append(f"    {line}")
                else:
                    lines.append(line)
        lines += self.translate_to_write_arrays(write - atomic)
        return stripped_deindented_lines("\n".join(lines))


class B200CodeObject(CPPStandaloneCodeObject):
    """A step-loop code object: carries its translated snippets, runs nothing on its own."""

    generator_class = B200CodeGenerator
    class_name = "b200_cuda"

    def __init__(self, owner, fragment, variables, variable_indices, template_name, name):
        super().__init__(owner, "", variables, variable_indices, template_name=template_name,
                         template_source="", name=name, compiler_kwds={})
        self.fragment = fragment

    def compile_block(self, block):
        pass

    def run_block(self, block):
        # executed inside the device step kernel; run on its own (outside a
        # network run, e.g. StateMonitor.record_single_timestep) it has no place
        if block == "run":
            raise NotImplementedError(f"b200: running the code object {self.name} outside run() is not supported")


class B200Device(CPPStandaloneDevice):
    """Standalone device whose clock-driven step loop runs on one GB300."""

    def __init__(self):
        super().__init__()
        self.b200_runs = []            # [(net, n_steps, spec, objects)]
        self.b200_run_options = dict(threads=None, ctas_per_inst=None)
        self.b200_last_network = None
        self.b200_timings = []
        self.b200_job_dir = None
        self.b200_report_kind = None   # the runs' progress report (one kind per device, as the reference)

    def reinit(self):
        opts = self.b200_run_options
        super().reinit()
        self.b200_runs = []
        self.b200_run_options = opts
        self.b200_last_network = None
        self.b200_timings = []
        self.b200_report_kind = None

    def activate(self, build_on_run=True, **kwargs):
        for k in ("threads", "ctas_per_inst"):
            if k in kwargs:
                self.b200_run_options[k] = kwargs.pop(k)
        super().activate(build_on_run=build_on_run, **kwargs)

    # ------------------------------------------------------------- code objects
    def code_object(self, owner, name, abstract_code, variables, template_name, variable_indices,
                    codeobj_class=None, template_kwds=None, override_conditional_write=None,
                    compiler_kwds=None):
        if template_name not in STEP_TEMPLATES:
            return super().code_object(owner, name, abstract_code, variables, template_name, variable_indices,
                                       codeobj_class=codeobj_class, template_kwds=template_kwds,
                                       override_conditional_write=override_conditional_write,
                                       compiler_kwds=compiler_kwds)
        from brian2.core.names import find_name
        name = find_name(name)
        meta = getattr(CPPStandaloneCodeObject.templater, template_name)
        for vname, var in variables.items():
            if isinstance(var, BinomialFunction):
                # a PoissonInput's binomial draws (a state update of its target group):
                # the device continues the reference's stream
                if template_name != "stateupdate":
                    raise NotImplementedError("b200: binomial functions in the step loop are only supported "
                                              "in PoissonInput")
                if prefs.devices.cpp_standalone.openmp_threads:
                    raise NotImplementedError("b200: PoissonInput needs openmp_threads = 0 (one generator stream)")
            if isinstance(var, Function) and vname in ("rand", "randn", "poisson") and vname in str(abstract_code):
                # rand()/randn() drawn once per neuron and step (PoissonGroup thresholds,
                # stochastic state updates): the device continues the reference's
                # stream; draws per spike or per synapse are not supported
                if not (vname in ("rand", "randn") and template_name in ("threshold", "stateupdate")):
                    raise NotImplementedError(f"b200: {vname}() in {template_name} code is not supported "
                                              "(random numbers in state updates and thresholds only)")
                if prefs.devices.cpp_standalone.openmp_threads:
                    raise NotImplementedError("b200: rand() in the step loop needs openmp_threads = 0 "
                                              "(one generator stream)")
        gen = B200CodeGenerator(variables=variables, variable_indices=variable_indices, owner=owner,
                                iterate_all=meta.iterate_all, codeobj_class=B200CodeObject,
                                override_conditional_write=override_conditional_write,
                                allows_scalar_write=meta.allows_scalar_write, name=name,
                                template_name=template_name)
        scalar_code, vector_code, kwds = gen.translate(abstract_code, dtype=prefs["core.default_float_dtype"])
        # functions other than Brian's default table (a TimedArray, a user
        # function) have no device implementation; they may come in through a
        # subexpression, so look for their calls in the generated code
        code_text = str(scalar_code) + str(vector_code)
        for vname, var in variables.items():
            if not isinstance(var, Function) or isinstance(var, BinomialFunction) or vname in DEFAULT_FUNCTIONS:
                continue
            try:
                impl = var.implementations[CPPCodeGenerator].name or vname
            except Exception:  # (no C++ implementation registered under this generator)
                impl = vname
            if re.search(r"\b(%s|%s)\s*\(" % (re.escape(vname), re.escape(impl)), code_text):
                raise NotImplementedError(f"b200: function '{vname}' in the step loop (Brian's default "
                                          "functions only)")
        fragment = dict(template=template_name, scalar=scalar_code, vector=vector_code,
                        vector_device=kwds.get("vector_code_device"), template_kwds=dict(template_kwds or {}),
                        variables=variables, variable_indices=variable_indices, generator=gen)
        codeobj = B200CodeObject(owner, fragment, variables, variable_indices, template_name, name)
        return codeobj

    # ------------------------------------------------------------- runs
    def network_run(self, net, duration, report=None, report_period=None, namespace=None, profile=None,
                    level=0, **kwds):
        from brian2.core.namespace import get_local_namespace
        if duration < 0:
            raise ValueError(f"Function 'run' expected a non-negative duration but got '{duration}'")
        # progress report (device.py:1842-1917): the standard reports are printed
        # by the job runner at the start and end of the run on the device
        if report is not None:
            if not isinstance(report, str):
                raise TypeError("report argument has to be either 'text', 'stdout', 'stderr', or the code for a "
                                "report function")
            if report not in ("text", "stdout", "stderr"):
                raise NotImplementedError("b200: report functions given as C++ code are not supported")
            kind = "stderr" if report == "stderr" else "stdout"
            if getattr(self, "b200_report_kind", None) not in (None, kind):
                raise NotImplementedError("The b200 device does not support multiple report functions, each run "
                                          "has to use the same (or none).")
            self.b200_report_kind = kind
        self.networks.add(net)
        self.enable_profiling = bool(profile)
        all_objects = net.sorted_objects
        net._clocks = {obj.clock for obj in all_objects}
        t_end = net.t + duration
        for clock in net._clocks:
            clock.set_interval(net.t, t_end)
        if namespace is None:
            namespace = get_local_namespace(level=level + 2)
        net.before_run(namespace)
        self.synapses |= {s for s in net.objects if isinstance(s, Synapses)}
        self.clocks.update(net._clocks)
        # one clock for the step loop; operations (run_regularly) may run on a
        # clock whose dt is a whole multiple of it
        if any(not hasattr(obj.clock, "dt_") for obj in all_objects):
            raise NotImplementedError("b200: event clocks are not supported")
        slower = lambda obj: type(obj) is CodeRunner or isinstance(obj, StateMonitor)
        main = {obj.clock for obj in all_objects if not slower(obj)}
        if len(main) != 1:
            raise NotImplementedError("b200: all objects of a network must share one clock "
                                      "(run_regularly operations and state monitors may use a multiple of its dt)")
        clock = next(iter(main))
        if self.b200_runs and self.b200_runs[0].get("dt", float(clock.dt_)) != float(clock.dt_):
            raise NotImplementedError("b200: the time step changed between runs")
        for obj in all_objects:
            if slower(obj) and obj.clock is not clock:
                k = float(obj.clock.dt_) / float(clock.dt_)
                if round(k) < 1 or abs(k - round(k)) > 1e-9 * k:
                    raise NotImplementedError(f"b200: {obj.name} runs every {k} steps (not a whole number)")
        n_steps = int(round(float(duration) / float(clock.dt_)))
        spec, objects = self._make_spec(net, all_objects, clock)
        if draws_random(spec) and not self.b200_runs:
            # the generator state where the step loop starts drawing (the C++
            # library's text form: 624 words and the position), then whether
            # randn() keeps a value and the value (a copy's randn() returns the
            # kept value without advancing its generator)
            self.main_queue.append(("insert_code",
                                    '{ std::ofstream _b200_rng(brian::results_dir + "b200_rng_state"); '
                                    '_b200_rng << brian::_random_generators[0]; '
                                    'brian::RandomGenerator _b200_c = brian::_random_generators[0], '
                                    '_b200_d = brian::_random_generators[0]; '
                                    'const double _b200_g = _b200_c.randn(); '
                                    'const int _b200_kept = _b200_c.rand() == _b200_d.rand() ? 1 : 0; '
                                    '_b200_rng << " " << _b200_kept << " " << std::hexfloat << _b200_g; }'))
        self.b200_runs.append(dict(net=net, n_steps=n_steps, spec=spec, objects=objects, clock=clock,
                                   dt=float(clock.dt_),
                                   report=None if report is None else ("stderr" if report == "stderr" else "stdout"),
                                   report_period=float(report_period) if report_period is not None else 10.0,
                                   queue_len=len(self.main_queue)))
        self.main_queue.append(("insert_code", f"// b200 network run {len(self.b200_runs) - 1} ({n_steps} steps)"))
        net.t_ = float(t_end)
        net.after_run()
        for c in net._clocks:
            self.array_cache[c.variables["timestep"]] = np.array([c._i_end])
            self.array_cache[c.variables["t"]] = np.array([c._i_end * c.dt_])
        if self.build_on_run:
            if self.has_been_run:
                raise RuntimeError("The network has already been built and run before. Use set_device with "
                                   "build_on_run=False and an explicit device.build call to use multiple "
                                   "run statements with this device.")
            self.build(direct_call=False, **self.build_options)

    def network_get_profiling_info(self, net):
        # (device.py:1991-2002: no information without profile=True; times as
        # quantities in seconds; one entry for the device's step loop)
        from brian2.units import second
        if not self.enable_profiling:
            raise ValueError("No profiling info collected (did you run with 'profile=True'?)")
        return sorted(((name, ms * 1e-3 * second) for name, ms in self.b200_timings), key=lambda x: -x[1])

    # ------------------------------------------------------------- spec
    def _make_spec(self, net, objects, clock):
        gen_name = CPPCodeGenerator.get_array_name
        groups, group_index = [], {}

        def group_of(g):
            base = g.source if isinstance(g, Subgroup) else g
            if not isinstance(base, (NeuronGroup, SpikeGeneratorGroup, PoissonGroup)):
                raise NotImplementedError(f"b200: unsupported source/target {g!r}")
            if base.name not in group_index:
                gv = []
                for vname, var in sorted(base.variables.items()):
                    if isinstance(base, SpikeGeneratorGroup) and vname != "i":
                        continue  # the spike lists are a generator's own arrays, not per-neuron state
                    if (isinstance(var, ArrayVariable) and not var.scalar and var.owner is not None
                            and var.owner.name == base.name and vname != "_spikespace"
                            and var.size == len(base) and getattr(var, "ndim", 1) == 1):
                        gv.append(dict(name=vname, ctype=c_data_type(var.dtype), ptr=gen_name(var)))
                group_index[base.name] = len(groups)
                groups.append(dict(name=base.name, vars=gv, _obj=base))
                if isinstance(base, SpikeGeneratorGroup):
                    groups[-1]["generator"] = True
            lo = g.start if isinstance(g, Subgroup) else 0
            hi = g.stop if isinstance(g, Subgroup) else len(base)
            return group_index[base.name], (int(lo), int(hi))

        def event_group_of(g, event):
            """The group whose spike list is the event's list: the group itself
            for 'spike'; for a custom event (NeuronGroup(events=...),
            groups/neurongroup.py:522-560) a shadow group on the same state
            arrays (alias_of), with the event's condition as its threshold and
            its run_on_event code as its reset, and no state update."""
            gi, rng = group_of(g)
            if event == "spike":
                return gi, rng
            if groups[gi].get("generator"):
                raise NotImplementedError("b200: custom events of a spike generator")
            key = groups[gi]["name"] + "\x00" + event
            if key not in group_index:
                group_index[key] = len(groups)
                groups.append(dict(name=f"{groups[gi]['name']}__{event}", vars=[dict(v) for v in groups[gi]["vars"]],
                                   alias_of=gi, event=event, _obj=groups[gi]["_obj"]))
            return group_index[key], rng

        clock_ptrs = dict(dt=gen_name(clock.variables["dt"]), t=gen_name(clock.variables["t"]),
                          timestep=gen_name(clock.variables["timestep"]))
        consts = {}

        def collect(frag, allowed_owners):
            """Constants used by a fragment; extra arrays of other groups."""
            extra = {}
            for vname, var in frag["variables"].items():
                if isinstance(var, Constant) and vname not in ("N", "_vectorisation_idx"):
                    consts.setdefault(vname, dict(name=vname, ctype=c_data_type(var.dtype),
                                                  value=float(var.value)))
                elif isinstance(var, ArrayVariable):
                    owner = var.owner
                    if owner is None or isinstance(owner, Clock) or owner.name in allowed_owners:
                        continue
                    if isinstance(owner, NeuronGroup) or isinstance(owner, Subgroup):
                        gi, _ = group_of(owner)
                        names = [v["name"] for v in groups[gi]["vars"]]
                        if vname in names or var.name in names:
                            extra[gen_name(var)] = ("group", gi, names.index(var.name))
            return extra

        def text(code):
            if isinstance(code, dict):
                code = code[None]
            if not isinstance(code, str):
                code = "\n".join(code)
            return code.strip("\n")

        def block(frag):
            out = dict(scalar=text(frag["scalar"]), vector=text(frag["vector"]))
            if frag.get("vector_device"):
                out["vector_device"] = text(frag["vector_device"])
            return out

        pathways, spkmons, ratemons, statemons = [], [], [], []
        summed_frags = []
        input_frags = []  # PoissonInputs, in schedule order
        op_frags = []  # operations (run_regularly), in schedule order
        statemon_pos = []  # positions of the state monitors in the schedule
        draw_sites = []  # (position in the schedule, site, the block or input whose code draws)
        b200_objects = []
        push_names = {}  # pathway -> its push code object (for the profile)
        syn_frags = []  # per-synapse code (clock-driven equations, run_regularly) and monitors of Synapses
        for pos, obj in enumerate(objects):
            if not obj.active:
                continue
            for co in obj._code_objects:
                if not isinstance(co, B200CodeObject):
                    continue
                frag = co.fragment
                t = frag["template"]
                b200_objects.append((obj, co))
                if not isinstance(obj, PoissonInput) and any(
                        isinstance(v, BinomialFunction) for v in frag["variables"].values()):
                    raise NotImplementedError("b200: binomial functions outside PoissonInput")
                if isinstance(obj, PoissonInput):
                    input_frags.append((obj, frag, pos))
                elif t in ("stateupdate", "statemonitor") and isinstance(
                        getattr(obj, "source" if t == "statemonitor" else "group", None), Synapses):
                    syn_frags.append((obj, frag, pos, t, co.name))
                elif type(obj) is CodeRunner and t == "stateupdate":
                    op_frags.append((obj, frag, pos))
                elif t in ("stateupdate", "threshold", "reset"):
                    gi, _ = event_group_of(obj.group, getattr(obj, "event", "spike") if t != "stateupdate" else "spike")
                    g = groups[gi]
                    key = {"stateupdate": "update"}.get(t, t)
                    b = block(frag)
                    ex = collect(frag, {g["name"]})
                    if ex:
                        b["extra_ptrs"] = {k: list(v) for k, v in ex.items()}
                    if t in ("threshold", "stateupdate"):
                        kinds = [k for k in ("rand", "randn") if f"_{k}(" in b["vector"]]
                        if len(kinds) > 1:
                            raise NotImplementedError("b200: rand() and randn() in one code object")
                        if kinds:
                            if prefs.devices.cpp_standalone.openmp_threads:
                                raise NotImplementedError("b200: random numbers in the step loop need "
                                                          "openmp_threads = 0 (one generator stream)")
                            _, calls = _draw_calls(b["vector"], kinds[0])
                            draw_sites.append((pos, dict(name=obj.name, kind=kinds[0], group=gi, lo=0, hi=-1,
                                                         calls=calls), b))
                    if t == "threshold":
                        b["refractory"] = bool(frag["template_kwds"].get("_uses_refractory", False))
                    if t == "reset":
                        g["_reset_pos"] = pos  # (the resets of a group and its events run in schedule order)
                    if key in g:
                        raise NotImplementedError(f"b200: several {t} code objects for one group")
                    b["_co"] = co.name  # (for the profile: the time of each code object)
                    g[key] = b
                elif t == "synapses":
                    pw = obj
                    if not isinstance(pw, SynapticPathway) or pw.prepost not in ("pre", "post"):
                        raise NotImplementedError("b200: unsupported synaptic pathway")
                    syn = pw.synapses
                    sgi, srange = event_group_of(pw.source, pw.event)
                    tgi, trange = group_of(pw.target)
                    sv, seen = [], set()
                    used = {id(v) for v in frag["variables"].values()}
                    for vname, var in sorted(syn.variables.items()):
                        if (isinstance(var, DynamicArrayVariable) and var.owner is not None
                                and var.owner.name == syn.name and getattr(var, "ndim", 1) == 1
                                and var.name not in ("_synaptic_pre", "_synaptic_post", "N_incoming", "N_outgoing")
                                and not var.scalar and id(var) in used and var.name not in seen):
                            seen.add(var.name)
                            sv.append(dict(name=var.name, ctype=c_data_type(var.dtype), ptr=gen_name(var)))
                    gptrs = {}
                    for vname, var in frag["variables"].items():
                        if isinstance(var, ArrayVariable) and var.owner is not None and \
                                isinstance(var.owner, (NeuronGroup, Subgroup)):
                            gi, _ = group_of(var.owner)
                            names = [v["name"] for v in groups[gi]["vars"]]
                            if var.name in names:
                                gptrs[gen_name(var)] = [gi, names.index(var.name)]
                    collect(frag, {syn.name, groups[sgi]["name"], groups[tgi]["name"]})
                    pathways.append(dict(name=pw.name, src=sgi, tgt=tgi, vars=sv,
                                         pre_ptr=gen_name(syn.variables["_synaptic_pre"]),
                                         post_ptr=gen_name(syn.variables["_synaptic_post"]),
                                         group_ptrs=gptrs, on_pre=block(frag),
                                         _obj=pw, _src_range=srange, _tgt_range=trange, _syn=syn.name,
                                         _co=co.name))
                    if pw.prepost == "post":  # spiking side = the postsynaptic neurons
                        pathways[-1]["prepost"] = "post"
                elif t == "synapses_push_spikes":
                    push_names[id(obj)] = co.name
                elif t == "spikegenerator":
                    group_of(obj)
                elif t == "spikemonitor":
                    if not isinstance(obj, EventMonitor):
                        raise NotImplementedError("b200: unsupported spike monitor")
                    gi, rng = event_group_of(obj.source, obj.event)
                    # the monitor's slot in the schedule (core/network.py:42-50):
                    # after its group's thresholder; recorded variables only
                    # before the step's deliveries, where they are the values
                    # the thresholder saw
                    base = obj.source.source if isinstance(obj.source, Subgroup) else obj.source
                    thr = getattr(base, "thresholder", {}).get(obj.event) if hasattr(base, "thresholder") else None
                    late = ("synapses", "after_synapses", "before_resets", "resets", "after_resets",
                            "before_end", "end")
                    if not (obj.when in ("after_thresholds", "before_synapses") + late or
                            (obj.when == "thresholds" and (thr is None or obj.order > thr.order))):
                        raise NotImplementedError(f"b200: a spike monitor in the '{obj.when}' slot before its "
                                                  "group's thresholder")
                    # recorded variables (monitors/spikemonitor.py:62-67): state
                    # variables of the monitored group, their values at the spike
                    extra = [v for v in obj.record_variables if v not in ("i", "t")]
                    if extra and obj.when in late:
                        raise NotImplementedError(f"b200: a spike monitor recording variables in the '{obj.when}' "
                                                  "slot (after the step's deliveries)")
                    names = [v["name"] for v in groups[gi]["vars"]]
                    if extra and groups[gi].get("generator"):
                        raise NotImplementedError("b200: a spike generator's monitor records i and t only")
                    for v in extra:
                        if v not in names:
                            raise NotImplementedError(f"b200: spike monitor recording '{v}' (not a state variable)")
                    if len(extra) > 8:
                        raise NotImplementedError("b200: a spike monitor recording more than 8 variables")
                    spkmons.append(dict(name=obj.name, group=gi, vars=[names.index(v) for v in extra], _obj=obj,
                                        _range=rng, _co=co.name, _vars=extra))
                elif t == "ratemonitor":
                    gi, rng = group_of(obj.source)
                    ratemons.append(dict(name=obj.name, group=gi, _obj=obj, _range=rng, _co=co.name))
                elif t == "statemonitor":
                    statemon_pos.append((pos, obj.when))
                    if obj.when not in ("start", "end"):
                        raise NotImplementedError("b200: state monitors record in the start or end slot")
                    gi, rng = group_of(obj.source)
                    names = [v["name"] for v in groups[gi]["vars"]]
                    for v in obj.record_variables:
                        if v not in names:
                            raise NotImplementedError(f"b200: recording '{v}' (not a state variable)")
                    statemons.append(dict(name=obj.name, group=gi, _obj=obj, _range=rng, when=obj.when,
                                          every=int(round(float(obj.clock.dt_) / float(clock.dt_))),
                                          _vars=list(obj.record_variables)))
                elif t == "summed_variable":
                    summed_frags.append((obj, frag))

        def synaptic_vars(syn, frag):
            used = {id(v) for v in frag["variables"].values()}
            out = []
            for vname, var in sorted(syn.variables.items()):
                if (isinstance(var, DynamicArrayVariable) and var.owner is not None
                        and var.owner.name == syn.name and getattr(var, "ndim", 1) == 1
                        and var.name not in ("_synaptic_pre", "_synaptic_post", "N_incoming", "N_outgoing")
                        and not var.scalar and id(var) in used and var.name not in {v["name"] for v in out}):
                    out.append(dict(name=var.name, ctype=c_data_type(var.dtype), ptr=gen_name(var)))
            return out

        def neuron_ptrs(frag):
            gptrs = {}
            for vname, var in frag["variables"].items():
                if isinstance(var, ArrayVariable) and var.owner is not None and \
                        isinstance(var.owner, (NeuronGroup, Subgroup)):
                    gi, _ = group_of(var.owner)
                    names = [v["name"] for v in groups[gi]["vars"]]
                    if var.name in names:
                        gptrs[gen_name(var)] = [gi, names.index(var.name)]
            return gptrs

        # summed variables (templates/summed_variable.cpp): they run over the
        # synapses of their Synapses object, held by its on_pre pathway or, for a
        # Synapses object without one, by a pathway that delivers no events
        summed = []
        for obj, frag in summed_frags:
            syn = obj.group
            tkw = frag["template_kwds"]
            tgi, _ = group_of(obj.target)
            tnames = [v["name"] for v in groups[tgi]["vars"]]
            if tkw["_target_var"].name not in tnames:
                raise NotImplementedError("b200: summed variable target is not a state variable")
            pi = next((k for k, p in enumerate(pathways) if p["_syn"] == syn.name), None)
            if pi is not None and pathways[pi].get("prepost") == "post":
                raise NotImplementedError("b200: summed variables of a Synapses object with on_post only")
            if pi is None:
                sgi, srange = group_of(syn.source)
                tg2, trange = group_of(syn.target)
                pathways.append(dict(name=syn.name + "_synapses", src=sgi, tgt=tg2, vars=[],
                                     pre_ptr=gen_name(syn.variables["_synaptic_pre"]),
                                     post_ptr=gen_name(syn.variables["_synaptic_post"]),
                                     group_ptrs={}, on_pre=dict(scalar="", vector=""), events=False,
                                     _obj=syn, _src_range=srange, _tgt_range=trange, _syn=syn.name))
                pi = len(pathways) - 1
            names = {v["name"] for v in pathways[pi]["vars"]}
            pathways[pi]["vars"] += [v for v in synaptic_vars(syn, frag) if v["name"] not in names]
            collect(frag, {syn.name} | {g["name"] for g in groups})
            summed.append(dict(name=obj.name, pathway=pi, tgt_group=tgi,
                               tgt_var=tnames.index(tkw["_target_var"].name),
                               index_post=tkw["_index_var"].name == "_synaptic_post",
                               group_ptrs=neuron_ptrs(frag), code=block(frag)))
        # per-synapse code of a Synapses object (its clock-driven equations,
        # synapses.py:779-794, and run_regularly operations) and state monitors
        # recording its variables: over its synapses, held by its first pathway or
        # by a pathway that delivers no events
        def syn_pathway(syn):
            pi = next((k for k, p in enumerate(pathways) if p["_syn"] == syn.name), None)
            if pi is None:
                sgi, srange = group_of(syn.source)
                tg2, trange = group_of(syn.target)
                pathways.append(dict(name=syn.name + "_synapses", src=sgi, tgt=tg2, vars=[],
                                     pre_ptr=gen_name(syn.variables["_synaptic_pre"]),
                                     post_ptr=gen_name(syn.variables["_synaptic_post"]),
                                     group_ptrs={}, on_pre=dict(scalar="", vector=""), events=False,
                                     _obj=syn, _src_range=srange, _tgt_range=trange, _syn=syn.name))
                pi = len(pathways) - 1
            return pi

        synops = []
        for obj, frag, pos, t, co_name in syn_frags:
            syn = obj.source if t == "statemonitor" else obj.group
            pi = syn_pathway(syn)
            every = int(round(float(obj.clock.dt_) / float(clock.dt_)))
            if abs(every * float(clock.dt_) - float(obj.clock.dt_)) > 1e-9 * float(clock.dt_):
                raise NotImplementedError(f"b200: {obj.name} runs every {float(obj.clock.dt_)} s (not a whole "
                                          "number of steps)")
            if obj.when not in ("start", "groups", "end") or (t == "statemonitor" and obj.when == "groups"):
                raise NotImplementedError(f"b200: {obj.name} in the '{obj.when}' slot (synaptic code and monitors "
                                          "run in the start, groups (code) and end slots)")
            if t == "statemonitor":
                names = list(obj.record_variables)
                own = {v["name"] for v in synaptic_vars(syn, {"variables": {k: syn.variables[k] for k in names
                                                                            if k in syn.variables}})}
                for v in names:
                    if v not in own:
                        raise NotImplementedError(f"b200: recording '{v}' of {syn.name} (not a synaptic variable)")
                have = {v["name"] for v in pathways[pi]["vars"]}
                pathways[pi]["vars"] += [dict(name=v, ctype=c_data_type(syn.variables[v].dtype),
                                              ptr=gen_name(syn.variables[v])) for v in sorted(own - have)]
                statemons.append(dict(name=obj.name, group=-1, syn=pi, _obj=obj, _range=(0, 0), when=obj.when,
                                      every=every, _vars=names, pos=pos))
                continue
            b = block(frag)
            if "_rand(" in b["vector"] or "_randn(" in b["vector"] or b.get("vector_device"):
                raise NotImplementedError(f"b200: random numbers in the per-synapse code of {syn.name}")
            if neuron_ptrs(frag) or collect(frag, {syn.name}):
                raise NotImplementedError(f"b200: per-synapse code of {syn.name} reading neuron variables")
            have = {v["name"] for v in pathways[pi]["vars"]}
            pathways[pi]["vars"] += [v for v in synaptic_vars(syn, frag) if v["name"] not in have]
            synops.append(dict(name=obj.name, pathway=pi, when=obj.when, every=every, code=b, _co=co_name, pos=pos))
        # Poisson inputs (brian2/input/poissoninput.py:20-141): a state update in the
        # synapses slot, after the on_pre pathways (order -1) and before the
        # on_post pathways (order +1), drawing one binomial count per neuron
        inputs = []
        for obj, frag, pos in input_frags:
            if obj.when != "synapses" or obj.order != 0:
                raise NotImplementedError("b200: PoissonInput runs in the synapses slot with order 0")
            fns = [v for v in frag["variables"].values() if isinstance(v, BinomialFunction)]
            if len(fns) != 1:
                raise NotImplementedError("b200: unsupported PoissonInput code")
            fn = fns[0]
            support = fn.implementations[CPPCodeGenerator].get_code(None)["support_code"]
            m, mn = _BINOM_RE.search(support), _NORMAL_RE.search(support)
            if m is not None:     # inversion (N*p <= 5 or N*(1-p) <= 5)
                qn, bound, n_str, P, Q, ret = m.groups()
                ret = ret.strip().replace(" ", "")
                if ret not in ("X", f"{n_str}-X"):
                    raise NotImplementedError("b200: unsupported binomial sampler")
                site = dict(name=obj.name, kind="binomial", lo=0, hi=-1, calls=1,
                            binom=dict(qn=qn, bound=bound, n=int(n_str), p=P, q=Q, reverse=ret != "X"))
            elif mn is not None:  # normal approximation: (float)(randn()*scale + loc)
                site = dict(name=obj.name, kind="binormal", lo=0, hi=-1, calls=1,
                            binom=dict(scale=mn.group(1), loc=mn.group(2)))
            else:
                raise NotImplementedError("b200: unsupported binomial sampler")
            gi, (lo, hi) = group_of(obj.group)
            g = groups[gi]
            b = block(frag)
            k = len(inputs)
            vec = b["vector"]
            if vec.count(fn.name + "(") != 1 or b.get("vector_device"):
                raise NotImplementedError("b200: unsupported PoissonInput code")
            vec = re.sub(r"\b%s\(" % re.escape(fn.name), "_b200_binomial(", vec)
            whole = not isinstance(obj.group, Subgroup)
            if not whole:  # the subgroup's index array is the contiguous range itself
                sub = gen_name(obj.group.variables["_sub_idx"])
                vec = re.sub(re.escape(sub) + r"\s*\[\s*_idx\s*\]", "_b200_abs_idx", vec)
            names = {v["ptr"] for v in g["vars"]}
            for ptr in set(re.findall(r"_ptr_array_\w+", vec + b["scalar"])):
                if ptr not in names and ptr not in clock_ptrs.values():
                    raise NotImplementedError(f"b200: PoissonInput code reads {ptr} (not a state variable "
                                              "of its target group)")
            if collect(frag, {g["name"]}):
                raise NotImplementedError("b200: PoissonInput reads another group's variables")
            tv = g["vars"][[v["name"] for v in g["vars"]].index(obj.target_var)]["ptr"] \
                if obj.target_var in [v["name"] for v in g["vars"]] else None
            for p in pathways:
                if p.get("prepost") == "post" and tv in p.get("group_ptrs", {}):
                    raise NotImplementedError("b200: PoissonInput into a variable an on_post pathway writes")
            for sm in summed:
                if sm["tgt_group"] == gi and g["vars"][sm["tgt_var"]]["ptr"] == tv:
                    raise NotImplementedError("b200: PoissonInput into a summed variable")
            inputs.append(dict(name=obj.name, group=gi, lo=int(lo), hi=-1 if whole else int(hi),
                               code=dict(scalar=b["scalar"], vector=vec)))
            site.update(group=gi, lo=int(lo), hi=-1 if whole else int(hi))
            draw_sites.append((pos, site, inputs[-1]))
        if len(inputs) > 8:
            raise NotImplementedError("b200: more than 8 PoissonInputs")
        # operations (Group.run_regularly, brian2/groups/group.py CodeRunner with
        # the stateupdate template): in the start slot before the state monitors,
        # or in the end slot after the resets; every k-th step of the network
        # clock (their code reads the group's clock: t and dt of the step)
        for obj, frag, pos in op_frags:
            if obj.when not in ("start", "end"):
                raise NotImplementedError(f"b200: run_regularly in the '{obj.when}' slot (start and end only)")
            if any(p_ < pos and w_ == obj.when for p_, w_ in statemon_pos):
                raise NotImplementedError(f"b200: run_regularly after a state monitor in the {obj.when} slot")
            gi, (lo, hi) = group_of(obj.group)
            g = groups[gi]
            b = block(frag)
            if "_rand(" in b["vector"] or "_randn(" in b["vector"] or b.get("vector_device"):
                raise NotImplementedError("b200: random numbers in run_regularly code")
            vec = b["vector"]
            whole = not isinstance(obj.group, Subgroup)
            if not whole:
                sub = gen_name(obj.group.variables["_sub_idx"])
                vec = re.sub(re.escape(sub) + r"\s*\[\s*_idx\s*\]", "_b200_abs_idx", vec)
            names = {v["ptr"] for v in g["vars"]}
            for ptr in set(re.findall(r"_ptr_array_\w+", vec + b["scalar"])):
                if ptr not in names and ptr not in clock_ptrs.values():
                    raise NotImplementedError(f"b200: run_regularly code reads {ptr} (not a state variable of "
                                              "its group)")
            if collect(frag, {g["name"]}):
                raise NotImplementedError("b200: run_regularly code reads another group's variables")
            every = int(round(float(obj.clock.dt_) / float(clock.dt_)))
            g.setdefault("ops", []).append(dict(name=obj.name, when=obj.when, every=every, lo=int(lo),
                                                hi=-1 if whole else int(hi),
                                                code=dict(scalar=b["scalar"], vector=vec)))
        # draw sites in the order of the schedule (the order of the draws); each
        # call of the site's code becomes _b200_draw_<site>_<call>(index)
        draws = []
        for _, site, holder in sorted(draw_sites, key=lambda x: x[0]):
            si = len(draws)
            code = holder["code"]["vector"] if "code" in holder else holder["vector"]
            if site["kind"] in ("rand", "randn"):
                name = "_" + site["kind"] + "("
                parts = code.split(name)
                code = parts[0] + "".join(f"_b200_draw_{si}_{c}(" + rest for c, rest in enumerate(parts[1:]))
            else:
                code = code.replace("_b200_binomial(", f"_b200_draw_{si}_0(")
                holder["draw"] = si
            if "code" in holder:
                holder["code"]["vector"] = code
            else:
                holder["vector"] = code
                holder["draw"] = si
            draws.append(site)
        if len(draws) > 8:
            raise NotImplementedError("b200: more than 8 code objects drawing random numbers")
        # pathways of one Synapses object (on_pre and on_post) share its synapses and
        # synaptic variables: the first one in schedule order owns them, the others
        # alias it; all carry the union of the variables their code uses
        by_syn = {}
        for pi, p in enumerate(pathways):
            by_syn.setdefault(p["_syn"], []).append(pi)
        for pis in by_syn.values():
            if len(pis) < 2:
                continue
            union = {}
            for pi in pis:
                for v in pathways[pi]["vars"]:
                    union.setdefault(v["name"], v)
            allv = [union[k] for k in sorted(union)]
            for pi in pis:
                pathways[pi]["vars"] = [dict(v) for v in allv]
            for pi in pis[1:]:
                pathways[pi]["alias"] = pis[0]
        for g in groups:
            for k in ("update", "threshold", "reset"):
                g.setdefault(k, None)
        # a group's resets and its custom events' resets (run_on_event) change the
        # same state: they run one after another in the schedule's order
        for gi, g in enumerate(groups):
            members = [gi] + [k for k, h in enumerate(groups) if h.get("alias_of") == gi]
            if len(members) > 1:
                with_reset = [k for k in members if groups[k]["reset"] is not None]
                g["reset_order"] = sorted(with_reset, key=lambda k: groups[k]["_reset_pos"])
        # every array pointer used by a group block must be declared: add the
        # clock and constant names used in snippets as they are
        fdt = prefs["core.default_float_dtype"]
        for p in pathways:
            if p.get("events", True) and id(p["_obj"]) in push_names:
                p["_push_co"] = push_names[id(p["_obj"])]
        spec = dict(name=f"{net.name}", float=c_data_type(fdt), consts=sorted(consts.values(), key=lambda c: c["name"]),
                    groups=groups, pathways=pathways, spike_monitors=spkmons, rate_monitors=ratemons,
                    state_monitors=statemons, clock_ptrs=clock_ptrs)
        if summed:
            spec["summed"] = summed
        if synops:
            if summed:
                raise NotImplementedError("b200: per-synapse code together with summed variables")
            spec["syn_ops"] = synops
        if draws:
            spec["draws"] = draws
        # every array the code of the step loop names must be one the device
        # holds (a shared variable, e.g. `s : 1 (shared)`, is not carried)
        known = set(clock_ptrs.values())
        for g in groups:
            known |= {v["ptr"] for v in g["vars"]}
        for p in pathways:
            known |= {v["ptr"] for v in p["vars"]} | {p["pre_ptr"], p["post_ptr"]}
        texts = [json.dumps({k: v for k, v in g.items() if k != "_obj"}) for g in groups]
        texts += [json.dumps(p["on_pre"]) for p in pathways] + [json.dumps(sm["code"]) for sm in summed]
        texts += [json.dumps(inp["code"]) for inp in inputs]
        for ptr in set(re.findall(r"_ptr_array_\w+", "\n".join(texts))):
            if ptr not in known:
                raise NotImplementedError(f"b200: the step loop reads {ptr}, which the device does not hold "
                                          "(a shared or another object's variable)")
        if inputs:
            spec["inputs"] = inputs
        return spec, b200_objects

    PRIVATE_KEYS = {"_obj", "_range", "_src_range", "_tgt_range", "_vars", "_syn", "_co", "_push_co"}

    @staticmethod
    def public_spec(spec):
        """The JSON-serialisable part of a spec (drops the Brian objects)."""
        def clean(x):
            if isinstance(x, dict):
                return {k: clean(v) for k, v in x.items() if k not in B200Device.PRIVATE_KEYS}
            if isinstance(x, list):
                return [clean(v) for v in x]
            if isinstance(x, tuple):
                return [clean(v) for v in x]
            return x
        return clean(spec)

    # ------------------------------------------------------------- build + GPU
    def build(self, directory="output", results_directory="results", compile=True, run=True, debug=False,
              clean=False, with_output=True, additional_source_files=None, run_args=None, direct_call=True,
              **kwds):
        for k in ("threads", "ctas_per_inst"):
            if k in kwds:
                self.b200_run_options[k] = kwds.pop(k)
        if "b200_defer" in kwds:
            self.b200_run_options["defer"] = bool(kwds.pop("b200_defer"))
        # host code after the first GPU run cannot run in `main` (before the GPU
        # runs); assignments of values to state and synaptic variables become
        # actions of the job, applied after the run they follow
        self.b200_actions = []
        if self.b200_runs:
            self.b200_actions = self._b200_take_actions()
        super().build(directory=directory, results_directory=results_directory, compile=compile, run=run,
                      debug=debug, clean=clean, with_output=with_output,
                      additional_source_files=additional_source_files, run_args=run_args,
                      direct_call=direct_call, **kwds)
        if run and self.b200_runs:
            self._run_on_gpu()

    def _load(self, var):
        fname = os.path.join(self.results_dir, self.get_array_filename(var))
        return np.fromfile(fname, dtype=var.dtype)

    def _b200_take_actions(self):
        """Takes the assignments of values to neuron-group state variables
        queued after the first run out of `main`'s queue (the reference's forms:
        device.py:440-545) and returns them as job actions: (after run k, kind,
        object, variable, indices or None, values).  Any other host code there
        is refused."""
        spec0 = self.b200_runs[0]["spec"]
        arrays = {}
        for gi, g in enumerate(spec0["groups"]):
            for v in g["vars"]:
                arrays[v["ptr"][len("_ptr"):]] = ("group", gi, v["name"])
        # (synaptic variables are not among them: an owner-mode event carries its
        # synapse's values from the step it was pushed)
        clock_arrays = {p_[len("_ptr"):] for p_ in spec0["clock_ptrs"].values()}
        actions, run = [], -1
        for q in range(self.b200_runs[0]["queue_len"], len(self.main_queue)):
            func, args = self.main_queue[q]
            if func == "insert_code" and str(args).startswith("// b200 network run"):
                run = int(str(args).split()[4])
                continue
            if func == "set_by_single_value" and args[0] in clock_arrays:
                # (Network.run sets the clock where the next run starts: the
                # device's runs follow each other step by step)
                self.main_queue[q] = ("insert_code", f"// b200: {args[0]} = {args[2]} (the next run's start)")
                continue
            target = arrays.get(args[0]) if func in ("set_by_constant", "set_by_array", "set_by_single_value",
                                                     "set_array_by_array") else None
            if target is None:
                raise NotImplementedError("b200: host code between or after run() calls is not supported "
                                          f"(found '{func}')")
            if func == "set_by_constant":
                index, values = None, np.asarray(args[1])
            elif func == "set_by_array":
                index, values = None, np.asarray(self.static_arrays[args[1]])
            elif func == "set_by_single_value":
                txt = str(args[2]).strip()
                val = {"true": 1.0, "false": 0.0}.get(txt.lower(), None)
                index, values = np.asarray([int(args[1])]), np.asarray([float(txt) if val is None else val])
            else:
                index, values = np.asarray(self.static_arrays[args[1]]), np.asarray(self.static_arrays[args[2]])
            actions.append((run, *target, index, values))
            self.main_queue[q] = ("insert_code", f"// b200: {func} {args[0]} applied after run {run} on the device")
        return actions

    def _store(self, var, values):
        fname = os.path.join(self.results_dir, self.get_array_filename(var))
        np.ascontiguousarray(values, dtype=var.dtype).tofile(fname)
        # the results file is now the value (get_value answers from the cache
        # first, e.g. the zeros a monitor's counts were created with)
        self.array_cache.pop(var, None)

    def b200_export_job(self, directory):
        """Writes the recorded runs as a job directory (:mod:`brian2_gb300.job`):
        the spec and the initial state that the standalone ``main`` wrote."""
        from .job import write_job
        spec0 = self.b200_runs[0]["spec"]
        pub = self.public_spec(spec0)
        for r in self.b200_runs[1:]:
            if r["spec"] is not spec0 and self.public_spec(r["spec"]) != pub:
                raise NotImplementedError("b200: the network changed between runs")
        clock = self.b200_runs[0]["clock"]
        dt = float(clock.dt_)
        init = {}
        for gi, g in enumerate(spec0["groups"]):
            init[f"g{gi}_N"] = np.int64(len(g["_obj"]))
            for v in g["vars"] if g.get("alias_of") is None else []:  # (a custom event's group shares them)
                init[f"g{gi}_{v['name']}"] = self._load(g["_obj"].variables[v["name"]])
            if g.get("generator"):
                gv = g["_obj"].variables
                init[f"g{gi}_gen_bins"] = self._load(gv["_timebins"]).astype(np.int32)
                init[f"g{gi}_gen_index"] = self._load(gv["neuron_index"]).astype(np.int32)
                init[f"g{gi}_gen_period"] = np.int64(self._load(gv["_period_bins"])[0])
                init[f"g{gi}_gen_last"] = np.int64(self._load(gv["_lastindex"])[0])
        for pi, p in enumerate(spec0["pathways"]):
            pseudo = not p.get("events", True)  # (the Synapses object itself: no delivering pathway)
            syn = p["_obj"] if pseudo else p["_obj"].synapses
            # the spiking side and the other side (for an on_post pathway: the
            # postsynaptic and the presynaptic neurons)
            src_arr = syn.variables["_synaptic_pre"] if pseudo else p["_obj"].synapse_sources
            tgt_arr = syn.variables["_synaptic_post"] if pseudo else p["_obj"].synapse_targets
            init[f"p{pi}_pre"] = (self._load(src_arr).astype(np.int64) - p["_src_range"][0]).astype(np.int32)
            init[f"p{pi}_post"] = (self._load(tgt_arr).astype(np.int64) - p["_tgt_range"][0]).astype(np.int32)
            dvar = None if pseudo else p["_obj"].variables["delay"]
            d = np.zeros(1) if pseudo else self._load(dvar)
            if pseudo or dvar.scalar:
                init[f"p{pi}_scalar_delay"] = np.int64(int(float(d[0]) / dt + 0.5) if d.size else 0)
            else:
                init[f"p{pi}_scalar_delay"] = np.int64(0)
                init[f"p{pi}_delay_steps"] = (d / dt + 0.5).astype(np.int32)
            init[f"p{pi}_src_range"] = np.asarray(p["_src_range"], np.int64)
            init[f"p{pi}_tgt_range"] = np.asarray(p["_tgt_range"], np.int64)
            for v in p["vars"] if p.get("alias", -1) < 0 else []:  # (an alias shares its owner's)
                init[f"p{pi}_{v['name']}"] = self._load(syn.variables[v["name"]])
        for mi, m in enumerate(spec0["spike_monitors"]):
            init[f"sm{mi}_range"] = np.asarray(m["_range"], np.int64)
        for mi, m in enumerate(spec0["rate_monitors"]):
            init[f"rm{mi}_range"] = np.asarray(m["_range"], np.int64)
        for mi, m in enumerate(spec0["state_monitors"]):
            idx = self._load(m["_obj"].variables["_indices"]).astype(np.int32)
            init[f"stm{mi}_idx"] = idx + m["_range"][0]
            init[f"stm{mi}_vars"] = np.asarray(m["_vars"])
        init["ts0"] = np.int64(int(self._load(clock.variables["timestep"])[0]))
        if draws_random(spec0):
            with open(os.path.join(self.results_dir, "b200_rng_state")) as f:
                tok = f.read().split()
            if len(tok) != 627:
                raise RuntimeError("b200: unexpected generator state format")
            st = [int(x) for x in tok[:625]]
            init["rng_words"] = np.asarray(st[:624], np.uint32)
            init["rng_position"] = np.int64(st[624])
            init["rng_gauss"] = np.asarray([float(int(tok[625])), float.fromhex(tok[626])], np.float64)
        actions = []
        for j, (after, kind, obj, var, index, values) in enumerate(getattr(self, "b200_actions", [])):
            init[f"act{j}_values"] = values
            if index is not None:
                init[f"act{j}_index"] = index.astype(np.int64)
            actions.append(dict(after=int(after), kind=kind, obj=int(obj), var=var, indexed=index is not None))
        opts = dict(self.b200_run_options)
        if self.enable_profiling:  # run(profile=True): the device profile, per code object
            opts["profile"] = True
        if any(r.get("report") for r in self.b200_runs):  # run(report=...): printed by the job runner
            opts["reports"] = [r.get("report") for r in self.b200_runs]
            opts["report_periods"] = [r.get("report_period", 10.0) for r in self.b200_runs]
        write_job(directory, pub, init, [r["n_steps"] for r in self.b200_runs], dt, opts,
                  actions=actions)
        self.b200_job_dir = directory
        return directory

    def b200_import_results(self, directory=None):
        """Writes the outputs of a job run (``out.npz``) into the standalone
        results files, where ``get_value`` and the monitors read them."""
        directory = directory or self.b200_job_dir
        spec0 = self.b200_runs[0]["spec"]
        clock = self.b200_runs[0]["clock"]
        dt = float(clock.dt_)
        with np.load(os.path.join(directory, "out.npz")) as z:
            out = {k: z[k] for k in z.files}
        ts0 = int(out["ts0"])
        self.b200_timings = self._b200_profile(spec0, out) if "prof_names" in out else \
            [("b200_step_kernel", float(out["device_ms"]))]
        self._last_run_time = float(out["device_ms"]) * 1e-3
        self._last_run_completed_fraction = 1.0
        for gi, g in enumerate(spec0["groups"]):
            for v in g["vars"] if g.get("alias_of") is None else []:
                self._store(g["_obj"].variables[v["name"]], out[f"g{gi}_{v['name']}"])
            if g.get("generator"):
                self._store(g["_obj"].variables["_lastindex"], np.array([int(out[f"g{gi}_gen_last"])]))
        for pi, p in enumerate(spec0["pathways"]):
            syn = p["_obj"] if not p.get("events", True) else p["_obj"].synapses
            for v in p["vars"] if p.get("alias", -1) < 0 else []:
                self._store(syn.variables[v["name"]], out[f"p{pi}_{v['name']}"])
        for mi, m in enumerate(spec0["spike_monitors"]):
            i, ts, cnt = out[f"sm{mi}_i"], out[f"sm{mi}_ts"], out[f"sm{mi}_count"]
            mon = m["_obj"]
            lo, hi = m["_range"]
            self._store(mon.variables["count"], cnt[: hi - lo])
            self._store(mon.variables["N"], np.array([len(i)]))
            if mon.record:  # (record=False: no i and t, monitors/spikemonitor.py:127-128)
                self._store(mon.variables["i"], i)
                self._store(mon.variables["t"], ts.astype(np.float64) * dt)
            for k, v in enumerate(m.get("_vars", [])):  # recorded variables, in the variable's type
                self._store(mon.variables[v], out[f"sm{mi}_vals"][:, k].astype(mon.variables[v].dtype))
        for mi, m in enumerate(spec0["rate_monitors"]):
            c = out[f"rm{mi}_counts"]
            mon = m["_obj"]
            lo, hi = m["_range"]
            n = hi - lo
            rate = np.array([1.0 * x / dt / n for x in c], dtype=np.float64) if n else np.zeros(len(c))
            self._store(mon.variables["rate"], rate)
            self._store(mon.variables["t"], (ts0 + np.arange(len(c))).astype(np.float64) * dt)
            self._store(mon.variables["N"], np.array([len(c)]))
        for mi, m in enumerate(spec0["state_monitors"]):
            tr = out[f"stm{mi}_trace"]
            mon = m["_obj"]
            ev = int(m.get("every", 1))  # the monitor's clock: t = its time step * its dt
            first = -(-ts0 // ev)
            self._store(mon.variables["t"], (first + np.arange(tr.shape[0])).astype(np.float64) * float(mon.clock.dt_))
            for k, v in enumerate(m["_vars"]):
                self._store(mon.variables[v], tr[:, k, :])
                mon.variables[v].size = tr[:, k, :].shape
            self._store(mon.variables["N"], np.array([tr.shape[0]]))
        ts_end = int(out["ts_end"])
        self._store(clock.variables["timestep"], np.array([ts_end]))
        self._store(clock.variables["t"], np.array([ts_end * dt]))
        logger.debug(f"b200: {sum(r['n_steps'] for r in self.b200_runs)} steps in "
                     f"{float(out['device_ms']):.2f} ms (device)")

    @staticmethod
    def _b200_profile(spec, out):
        """(code object name, ms) from the device profile of a job run: the
        kernels' launch time split in proportion to the SM cycles of each
        profile slot (b200_get_profile), the slots mapped to the code objects
        they run -- a group's state updater, thresholder (its spike list) and
        resetter, a pathway's push (delay ring, delivery windows and items,
        shared equally by the pathways from one group) and its on_pre code, the
        monitors.  Time spent waiting at the instance barriers belongs to no
        code object and is left out, as the reference's profile covers code
        objects only (templates/common_group.cpp:72-90)."""
        names = [str(x) for x in out["prof_names"]]
        cyc = dict(zip(names, (float(x) for x in out["prof_cycles"])))
        total = sum(cyc.values())
        if total <= 0:
            return []
        ms_per = float(out["kernel_ms"]) / total
        t = {}

        def add(co, c):
            if co and c > 0:
                t[co] = t.get(co, 0.0) + c * ms_per
        owner = bool(int(out.get("owner", 0)))
        groups, paths = spec["groups"], spec["pathways"]
        deliv = [p for p in paths if p.get("events", True)]
        if owner:  # (the owner-mode kernel's coarser phases)
            for g in groups:
                add((g.get("update") or {}).get("_co"), cyc.get("update_threshold_reset", 0) / len(groups))
                add((g.get("threshold") or {}).get("_co"), cyc.get("spike_lists_monitors", 0) / len(groups))
            for p in deliv:
                add(p.get("_push_co"), (cyc.get("push_count", 0) + cyc.get("push_fifo", 0)) / len(deliv))
                add(p.get("_co"), cyc.get("deliver", 0) / len(deliv))
        else:
            for g in groups:
                for blk, slot in (("update", "update"), ("threshold", "threshold"), ("reset", "reset")):
                    add((g.get(blk) or {}).get("_co"), cyc.get(f"{slot}:{g['name']}", 0))
            for gi, g in enumerate(groups):
                out_p = [p for p in deliv if p["src"] == gi]
                for p in out_p:
                    add(p.get("_push_co"), cyc.get(f"ring:{g['name']}", 0) / len(out_p))
            for p in deliv:
                add(p.get("_push_co"), (cyc.get("delay_windows", 0) + cyc.get("items", 0)) / len(deliv))
            from .codegen import delivery_passes
            for _, pis, _ in delivery_passes(paths):  # a shared pass: its events split equally
                c = cyc.get(f"events:{paths[pis[0]]['name']}", 0)
                for q in pis:
                    add(paths[q].get("_co"), c / len(pis))
            for m in spec["spike_monitors"]:
                add(m.get("_co"), cyc.get(f"spikemon:{m['name']}", 0))
            for m in spec["rate_monitors"]:
                add(m.get("_co"), cyc.get(f"ratemon:{m['name']}", 0))
        return sorted(t.items(), key=lambda x: -x[1])

    def _run_on_gpu(self):
        """Export the runs as a job, run it on this host's GPU, import the
        results.  With ``build(..., b200_defer=True)`` only the job is written
        (to be run where the GPU is, then ``b200_import_results``)."""
        from .job import run_job
        directory = self.b200_export_job(os.path.join(self.project_dir, "b200_job"))
        if self.b200_run_options.get("defer"):
            logger.info(f"b200: job written to {directory}; run it with `python -m brian2_gb300.job "
                        f"{directory}` and import the results with device.b200_import_results()")
            return
        run_job(directory)
        self.b200_import_results(directory)


b200_device = B200Device()
all_devices["b200"] = b200_device
all_devices["gb300"] = b200_device
