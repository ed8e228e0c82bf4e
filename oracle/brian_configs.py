"""Workload definitions written as ordinary Brian2 scripts.

Test infrastructure only: these functions build the benchmark networks with the
reference Brian2 API so that (a) the oracle fixtures can be produced by Brian2's
own ``cpp_standalone`` device and (b) the ``b200`` device can be checked on the
very same scripts.  They need an importable ``brian2`` (see make_ref_env.sh).

Each builder takes the network size and simulated duration as arguments so the
same construction can be run at reduced sizes; it returns a dict of the
monitors it created.  The synapse construction calls follow
``brian2/synapses/synapses.py:1608-1741`` (``Synapses.connect``).
"""


def cuba(N=4000, duration_ms=1000.0, seed_value=1234, ne_frac=0.8, refractory=False):
    """CUBA: exact-linear LIF, exponential currents, Bernoulli p=0.02, no delays."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor,
                        ms, mV, seed, run)
    seed(seed_value)
    taum = 20 * ms; taue = 5 * ms; taui = 10 * ms
    Vt = -50 * mV; Vr = -60 * mV; El = -49 * mV
    eqs = '''
    dv/dt  = (ge+gi-(v-El))/taum : volt
    dge/dt = -ge/taue : volt
    dgi/dt = -gi/taui : volt
    '''
    Ne = int(N * ne_frac)
    P = NeuronGroup(N, eqs, threshold='v>Vt', reset='v = Vr', method='exact',
                    namespace=dict(taum=taum, taue=taue, taui=taui, Vt=Vt, Vr=Vr, El=El))
    P.v = 'Vr + rand() * (Vt - Vr)'
    we = (60 * 0.27 / 10) * mV
    wi = (-20 * 4.5 / 10) * mV
    Ce = Synapses(P, P, on_pre='ge += we', namespace=dict(we=we))
    Ci = Synapses(P, P, on_pre='gi += wi', namespace=dict(wi=wi))
    Ce.connect(f'i<{Ne} and i!=j', p=0.02)
    Ci.connect(f'i>={Ne} and i!=j', p=0.02)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, Ce=Ce, Ci=Ci, spikes=s_mon, rate=r_mon)


def cobahh(N=4000, duration_ms=1000.0, seed_value=1234, ne_frac=0.8):
    """COBAHH: Hodgkin-Huxley, conductance synapses, exponential_euler."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor,
                        Equations, ms, mV, nS, siemens, msiemens, ufarad, cm, umetre,
                        seed, run)
    seed(seed_value)
    area = 20000 * umetre ** 2
    ns = dict(
        Cm=(1 * ufarad * cm ** -2) * area, gl=(5e-5 * siemens * cm ** -2) * area,
        El=-60 * mV, EK=-90 * mV, ENa=50 * mV,
        g_na=(100 * msiemens * cm ** -2) * area, g_kd=(30 * msiemens * cm ** -2) * area,
        VT=-63 * mV, taue=5 * ms, taui=10 * ms, Ee=0 * mV, Ei=-80 * mV,
        we=6 * nS, wi=67 * nS)
    eqs = Equations('''
    dv/dt = (gl*(El-v)+ge*(Ee-v)+gi*(Ei-v)-
             g_na*(m*m*m)*h*(v-ENa)-
             g_kd*(n*n*n*n)*(v-EK))/Cm : volt
    dm/dt = alpha_m*(1-m)-beta_m*m : 1
    dn/dt = alpha_n*(1-n)-beta_n*n : 1
    dh/dt = alpha_h*(1-h)-beta_h*h : 1
    dge/dt = -ge*(1./taue) : siemens
    dgi/dt = -gi*(1./taui) : siemens
    alpha_m = 0.32*(mV**-1)*4*mV/exprel((13*mV-v+VT)/(4*mV))/ms : Hz
    beta_m = 0.28*(mV**-1)*5*mV/exprel((v-VT-40*mV)/(5*mV))/ms : Hz
    alpha_h = 0.128*exp((17*mV-v+VT)/(18*mV))/ms : Hz
    beta_h = 4./(1+exp((40*mV-v+VT)/(5*mV)))/ms : Hz
    alpha_n = 0.032*(mV**-1)*5*mV/exprel((15*mV-v+VT)/(5*mV))/ms : Hz
    beta_n = .5*exp((10*mV-v+VT)/(40*mV))/ms : Hz
    ''')
    Ne = int(N * ne_frac)
    P = NeuronGroup(N, model=eqs, threshold='v>-20*mV', refractory='v>-20*mV',
                    method='exponential_euler', namespace=ns)
    Ce = Synapses(P, P, on_pre='ge+=we', namespace=ns)
    Ci = Synapses(P, P, on_pre='gi+=wi', namespace=ns)
    Ce.connect(f'i<{Ne}', p=0.02)
    Ci.connect(f'i>={Ne}', p=0.02)
    P.v = 'El + (randn() * 5 - 5)*mV'
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, Ce=Ce, Ci=Ci, spikes=s_mon, rate=r_mon)


def cuba_delays(N=10000, K=1000, duration_ms=1000.0, seed_value=1234, ne_frac=0.8,
                wscale=1.0 / 50, dmin_ms=0.1, dmax_ms=5.0, warmup_ms=0.0, report=None, report_period_s=10.0):
    """Large CUBA: fixed in-degree K split 80/20 between E and I sources.

    Every neuron receives exactly ``ne_frac*K`` synapses from distinct sources
    drawn uniformly from the excitatory population and ``K - ne_frac*K`` from the
    inhibitory one (``sample(N_pre, size=...)`` per target).  Weights are a
    per-synapse variable ``w`` and delays are drawn uniformly per synapse.
    With ``warmup_ms`` a first ``run(warmup_ms)`` precedes the run of
    ``duration_ms``; ``report`` and ``report_period_s`` are passed to that run
    (Brian's progress report: for the standalone device, C++ code of the
    report function, ``device.py:1889-1907``).
    """
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor,
                        ms, mV, seed, run)
    seed(seed_value)
    taum = 20 * ms; taue = 5 * ms; taui = 10 * ms
    Vt = -50 * mV; Vr = -60 * mV; El = -49 * mV
    eqs = '''
    dv/dt  = (ge+gi-(v-El))/taum : volt
    dge/dt = -ge/taue : volt
    dgi/dt = -gi/taui : volt
    '''
    Ne = int(N * ne_frac)
    Ke = int(K * ne_frac)
    Ki = K - Ke
    P = NeuronGroup(N, eqs, threshold='v>Vt', reset='v = Vr', method='exact',
                    namespace=dict(taum=taum, taue=taue, taui=taui, Vt=Vt, Vr=Vr, El=El))
    P.v = 'Vr + rand() * (Vt - Vr)'
    ns = dict(we=(60 * 0.27 / 10) * mV * wscale, wi=(-20 * 4.5 / 10) * mV * wscale,
              dmin=dmin_ms * ms, dspan=(dmax_ms - dmin_ms) * ms)
    Ce = Synapses(P[:Ne], P, model='w : volt', on_pre='ge += w', namespace=ns)
    Ci = Synapses(P[Ne:], P, model='w : volt', on_pre='gi += w', namespace=ns)
    Ce.connect(i=f'k for k in sample(N_pre, size={Ke})')
    Ci.connect(i=f'k for k in sample(N_pre, size={Ki})')
    Ce.w = 'we'
    Ce.delay = 'dmin + rand()*dspan'
    Ci.w = 'wi'
    Ci.delay = 'dmin + rand()*dspan'
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    from brian2 import second
    if warmup_ms > 0:
        run(warmup_ms * ms)
    if report is None:
        run(duration_ms * ms)
    else:
        run(duration_ms * ms, report=report, report_period=report_period_s * second)
    return dict(P=P, Ce=Ce, Ci=Ci, spikes=s_mon, rate=r_mon)


def cuba_sweep(params, duration_ms=500.0, ne_frac=0.8, report=None):
    """Networks of a parameter sweep, one after another in one script: for each
    parameter set (``N``, ``seed``, ``taum`` in s, excitatory weight scale
    ``wscale``) the construction of ``cuba`` with that size, seed, membrane time
    constant and excitatory weight, built and run by its own ``Network``.  In
    the standalone device every ``seed``, construction and run is executed by
    ``main`` in script order, so each network is what ``cuba`` alone builds.
    ``report`` (standalone: C++ code of the report function) goes to every run;
    its end-of-run call gives each network's own run time
    (``templates/network.cpp:114-121``)."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, Network, ms, mV, second, seed
    out = []
    for p in params:
        seed(p["seed"])
        Vt = -50 * mV; Vr = -60 * mV; El = -49 * mV
        eqs = '''
        dv/dt  = (ge+gi-(v-El))/taum : volt
        dge/dt = -ge/taue : volt
        dgi/dt = -gi/taui : volt
        '''
        N = p["N"]
        Ne = int(N * ne_frac)
        P = NeuronGroup(N, eqs, threshold='v>Vt', reset='v = Vr', method='exact',
                        namespace=dict(taum=p["taum"] * second, taue=5 * ms, taui=10 * ms, Vt=Vt, Vr=Vr, El=El))
        P.v = 'Vr + rand() * (Vt - Vr)'
        Ce = Synapses(P, P, on_pre='ge += we', namespace=dict(we=(60 * 0.27 / 10) * mV * p["wscale"]))
        Ci = Synapses(P, P, on_pre='gi += wi', namespace=dict(wi=(-20 * 4.5 / 10) * mV))
        Ce.connect(f'i<{Ne} and i!=j', p=0.02)
        Ci.connect(f'i>={Ne} and i!=j', p=0.02)
        s_mon = SpikeMonitor(P)
        net = Network(P, Ce, Ci, s_mon)
        if report is None:
            net.run(duration_ms * ms)
        else:
            net.run(duration_ms * ms, report=report, report_period=1e6 * second)
        out.append(dict(P=P, Ce=Ce, Ci=Ci, spikes=s_mon))
    return out


# ---------------------------------------------------------------------------
# Scenarios beyond the benchmark networks (parity of less common step-loop
# features: timed refractoriness, heterogeneous weights and delays, monitors
# on subgroups, a state monitor, a separate input group, on_pre reading a
# presynaptic variable).  Each returns its monitors.
# ---------------------------------------------------------------------------
def lif_refractory(N=300, duration_ms=200.0, seed_value=11):
    """LIF driven by a per-neuron constant input, 2 ms refractory period
    (``v`` clamped while refractory), recurrent excitation p=0.05."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, ms, mV, seed, run
    seed(seed_value)
    ns = dict(tau=10 * ms, Vt=-50 * mV, Vr=-65 * mV, El=-65 * mV, w=0.4 * mV)
    P = NeuronGroup(N, '''dv/dt = (El - v + I)/tau : volt (unless refractory)
                          I : volt (constant)''',
                    threshold='v > Vt', reset='v = Vr', refractory=2 * ms, method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    P.I = '12*mV + rand() * 8*mV'
    S = Synapses(P, P, on_pre='v += w', namespace=ns)
    S.connect('i != j', p=0.05)
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, S=S, spikes=s_mon, rate=r_mon)


def hetero_delays(N=400, duration_ms=150.0, seed_value=21):
    """CUBA dynamics with per-synapse random weights and delays (0-3 ms)."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, ms, mV, seed, run
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-49 * mV)
    P = NeuronGroup(N, '''dv/dt  = (ge-(v-El))/taum : volt
                          dge/dt = -ge/taue : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    S = Synapses(P, P, model='w : volt', on_pre='ge += w', namespace=ns)
    S.connect('i != j', p=0.05)
    S.w = '(rand() - 0.3) * 1.5*mV'
    S.delay = 'rand() * 3*ms'
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, S=S, spikes=s_mon, rate=r_mon)


def subgroup_monitors(N=500, duration_ms=200.0, seed_value=31):
    """CUBA with monitors on parts of the group and a state monitor."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, StateMonitor,
                        ms, mV, seed, run)
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, taui=10 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-49 * mV,
              we=1.62 * mV, wi=-9 * mV)
    P = NeuronGroup(N, '''dv/dt  = (ge+gi-(v-El))/taum : volt
                          dge/dt = -ge/taue : volt
                          dgi/dt = -gi/taui : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    Ne = int(0.8 * N)
    Ce = Synapses(P[:Ne], P, on_pre='ge += we', namespace=ns)
    Ci = Synapses(P[Ne:], P, on_pre='gi += wi', namespace=ns)
    Ce.connect(p=0.02)
    Ci.connect(p=0.02)
    s_mon = SpikeMonitor(P[100:300])
    r_mon = PopulationRateMonitor(P[:50])
    st_mon = StateMonitor(P, 'v', record=[0, 10, 250, 499])
    run(duration_ms * ms)
    return dict(P=P, Ce=Ce, Ci=Ci, spikes=s_mon, rate=r_mon, state=st_mon)


def input_group(N_in=200, N=300, duration_ms=200.0, seed_value=41):
    """A separate group of driven input neurons projecting with delays onto a
    recurrent CUBA population."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, ms, mV, seed, run
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-60 * mV, w_in=2 * mV, w=0.5 * mV,
              tau_in=5 * ms)
    inp = NeuronGroup(N_in, '''dv/dt = (-60*mV - v + I)/tau_in : volt
                               I : volt (constant)''',
                      threshold='v > -50*mV', reset='v = -60*mV', method='exact', namespace=ns)
    inp.v = '-60*mV + rand() * 10*mV'
    inp.I = '8*mV + rand() * 6*mV'
    P = NeuronGroup(N, '''dv/dt  = (ge-(v-El))/taum : volt
                          dge/dt = -ge/taue : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    Sin = Synapses(inp, P, on_pre='ge += w_in', namespace=ns)
    Sin.connect(p=0.1)
    Sin.delay = '1*ms + rand() * 2*ms'
    S = Synapses(P, P, on_pre='ge += w', namespace=ns)
    S.connect('i != j', p=0.05)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, inp=inp, Sin=Sin, S=S, spikes=s_mon, rate=r_mon)


def presynaptic_read(N=300, duration_ms=150.0, seed_value=51):
    """on_pre uses a variable of the presynaptic neuron (its adaptation
    current at delivery time)."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, ms, mV, seed, run
    seed(seed_value)
    ns = dict(taum=15 * ms, taue=5 * ms, taua=50 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-48 * mV)
    P = NeuronGroup(N, '''dv/dt  = (ge-(v-El))/taum : volt
                          dge/dt = -ge/taue : volt
                          da/dt = -a/taua : 1''',
                    threshold='v>Vt', reset='v = Vr; a += 0.2', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    S = Synapses(P, P, on_pre='ge_post += 1.2*mV * (1 - a_pre)', namespace=ns)
    S.connect('i != j', p=0.05)
    S.delay = '0.5*ms'
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, S=S, spikes=s_mon, rate=r_mon)


def spike_generator(N_in=100, N=300, duration_ms=130.0, period_ms=40.0, seed_value=61):
    """A SpikeGeneratorGroup (four spikes per input in each 40 ms period,
    some at exact multiples of dt, repeated three and a quarter times) driving
    a recurrent CUBA population through synapses with delays."""
    import numpy as np
    from brian2 import (NeuronGroup, Synapses, SpikeGeneratorGroup, SpikeMonitor, PopulationRateMonitor,
                        ms, mV, seed, run)
    seed(seed_value)
    rng = np.random.default_rng(seed_value)
    n_bins = int(round(period_ms / 0.1))
    idx, times = [], []
    for k in range(N_in):
        bins = rng.choice(n_bins, size=4, replace=False)
        jitter = np.where(rng.random(4) < 0.25, 0.0, rng.random(4) * 0.09)
        idx.extend([k] * 4)
        times.extend(list(bins * 0.1 + jitter))
    G = SpikeGeneratorGroup(N_in, np.array(idx), np.array(times) * ms, period=period_ms * ms)
    ns = dict(taum=20 * ms, taue=5 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-52 * mV, w_in=3 * mV, w=0.5 * mV)
    P = NeuronGroup(N, '''dv/dt  = (ge-(v-El))/taum : volt
                          dge/dt = -ge/taue : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    Sin = Synapses(G, P, on_pre='ge += w_in', namespace=ns)
    Sin.connect(p=0.1)
    Sin.delay = 'rand() * 2*ms'
    S = Synapses(P, P, on_pre='ge += w', namespace=ns)
    S.connect('i != j', p=0.05)
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    g_mon = SpikeMonitor(G)
    run(duration_ms * ms)
    return dict(P=P, G=G, Sin=Sin, S=S, spikes=s_mon, rate=r_mon, gen_spikes=g_mon)


def stdp(N_in=200, N=50, duration_ms=300.0, rate_hz=15.0, seed_value=71):
    """Event-driven STDP (pair-based traces, additive, clipped) from a spike
    generator onto a small LIF population.  The on_pre and on_post pathways of
    the Synapses object share the weight, the traces and their last-update
    time; the on_pre pathway has random delays (0-2 ms), on_post none."""
    import numpy as np
    from brian2 import (NeuronGroup, Synapses, SpikeGeneratorGroup, SpikeMonitor, PopulationRateMonitor,
                        ms, mV, seed, run)
    seed(seed_value)
    rng = np.random.default_rng(seed_value)
    n_bins = int(round(duration_ms / 0.1))
    idx, times = [], []
    for k in range(N_in):  # independent Bernoulli trains at rate_hz, one spike per bin at most
        bins = np.nonzero(rng.random(n_bins) < rate_hz * 1e-4)[0]
        idx.extend([k] * len(bins))
        times.extend(list(bins * 0.1 + 0.05))
    order = np.argsort(times, kind="stable")
    G = SpikeGeneratorGroup(N_in, np.array(idx)[order], np.array(times)[order] * ms)
    ns = dict(taum=10 * ms, taue=5 * ms, Vt=-54 * mV, Vr=-60 * mV, El=-65 * mV, drive=15 * mV,
              taupre=20 * ms, taupost=20 * ms, wmax=1.0, dApre=0.01, dApost=-0.0105)
    P = NeuronGroup(N, '''dv/dt = (El - v + ge * drive)/taum : volt
                          dge/dt = -ge/taue : 1''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    S = Synapses(G, P, '''w : 1
                          dApre/dt = -Apre/taupre : 1 (event-driven)
                          dApost/dt = -Apost/taupost : 1 (event-driven)''',
                 on_pre='''ge_post += w
                           Apre += dApre
                           w = clip(w + Apost, 0, wmax)''',
                 on_post='''Apost += dApost
                            w = clip(w + Apre, 0, wmax)''', namespace=ns)
    S.connect(p=0.3)
    S.w = 'rand() * 0.5'
    S.delay = 'rand() * 2*ms'
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    g_mon = SpikeMonitor(G)
    run(duration_ms * ms)
    return dict(P=P, G=G, S=S, spikes=s_mon, rate=r_mon, gen_spikes=g_mon, syn_vars=("w", "Apre", "Apost"))


def gap_junctions(N=200, duration_ms=200.0, seed_value=81):
    """Electrically coupled LIF neurons: a summed variable (Igap_post = w *
    (v_pre - v_post), summed over each neuron's gap junctions every step) in a
    Synapses object without on_pre, plus chemical synapses with delays."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, StateMonitor, ms, seed, run
    seed(seed_value)
    ns = dict(tau=10 * ms, w_syn=0.05)
    P = NeuronGroup(N, '''dv/dt = (v0 - v + Igap) / tau : 1
                          v0 : 1 (constant)
                          Igap : 1''',
                    threshold='v > 1', reset='v = 0', method='exact', namespace=ns)
    P.v = 'rand()'
    P.v0 = '1.02 + rand() * 0.2'
    G = Synapses(P, P, '''w : 1 (constant)
                          Igap_post = w * (v_pre - v_post) : 1 (summed)''', namespace=ns)
    G.connect('i != j', p=0.05)
    G.w = 'rand() * 0.02'
    S = Synapses(P, P, on_pre='v_post += w_syn', namespace=ns)
    S.connect('i != j', p=0.02)
    S.delay = '1*ms + rand() * 2*ms'
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    st_mon = StateMonitor(P, ['v', 'Igap'], record=[0, 7, 150])
    run(duration_ms * ms)
    return dict(P=P, G=G, S=S, spikes=s_mon, rate=r_mon, state=st_mon, state_extra=("Igap",))


def explicit_methods(N=300, duration_ms=150.0, seed_value=91):
    """Nonlinear (quadratic integrate-and-fire with adaptation) neurons
    integrated with the explicit methods: one group with 'euler', one with
    'rk4' (stateupdaters/explicit.py), coupled by synapses with delays."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, ms, mV, seed, run
    seed(seed_value)
    ns = dict(tau=10 * ms, tau_w=100 * ms, El=-65 * mV, Vc=-50 * mV, Vr=-70 * mV, Vpeak=-30 * mV,
              a=0.2, b=2 * mV, kq=15 * mV, w_syn=1.5 * mV)
    eqs = '''dv/dt = ((v - El) * (v - Vc) / kq - u + I) / tau : volt
             du/dt = (a * (v - El) - u) / tau_w : volt
             I : volt (constant)'''
    P = NeuronGroup(N, eqs, threshold='v > Vpeak', reset='v = Vr; u += b', method='euler', namespace=ns)
    P.v = 'El + rand() * 5*mV'
    P.I = '10*mV + rand() * 8*mV'
    Q = NeuronGroup(N, eqs, threshold='v > Vpeak', reset='v = Vr; u += b', method='rk4', namespace=ns)
    Q.v = 'El + rand() * 5*mV'
    Q.I = '10*mV + rand() * 8*mV'
    S = Synapses(P, Q, on_pre='v_post += w_syn', namespace=ns)
    S.connect(p=0.05)
    S.delay = '0.5*ms + rand() * 1*ms'
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(Q)
    r_mon = PopulationRateMonitor(Q)
    p_mon = SpikeMonitor(P)
    run(duration_ms * ms)
    return dict(P=Q, G=P, spikes=s_mon, rate=r_mon, other_spikes=p_mon)


def poisson_input(N_in=300, N=200, duration_ms=200.0, seed_value=101):
    """A PoissonGroup (rates 5-45 Hz, a draw of the reference's generator per
    neuron and step) driving a CUBA population through synapses with delays;
    a second PoissonGroup at a uniform rate draws after it."""
    import numpy as np
    from brian2 import (NeuronGroup, PoissonGroup, Synapses, SpikeMonitor, PopulationRateMonitor,
                        ms, mV, Hz, seed, run)
    seed(seed_value)
    G = PoissonGroup(N_in, rates=(5 + 40 * np.arange(N_in) / N_in) * Hz)
    H = PoissonGroup(50, rates=30 * Hz)
    ns = dict(taum=20 * ms, taue=5 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-60 * mV, w_in=1.5 * mV, w_h=2 * mV)
    P = NeuronGroup(N, '''dv/dt  = (ge-(v-El))/taum : volt
                          dge/dt = -ge/taue : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    S = Synapses(G, P, on_pre='ge += w_in', namespace=ns)
    S.connect(p=0.1)
    S.delay = 'rand() * 2*ms'
    T = Synapses(H, P, on_pre='ge += w_h', namespace=ns)
    T.connect(p=0.2)
    # monitors must be locals of the frame that calls run() (Brian collects them there)
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    g_mon = SpikeMonitor(G)
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, other_spikes=g_mon)


def poisson_drive(N=400, duration_ms=200.0, seed_value=202):
    """Poisson inputs (binomial counts drawn from the reference's generator)
    into a recurrent CUBA population with delays: one into ge over the whole
    group, one into v of a subgroup with a weight read from a state variable
    (the reset follows it), one with rate*dt > 0.5 (the sampler's reversed
    form) into gi, after a pathway into gi; a PoissonGroup draws before them
    in every step."""
    from brian2 import (NeuronGroup, PoissonGroup, PoissonInput, Synapses, SpikeMonitor, PopulationRateMonitor,
                        StateMonitor, ms, mV, Hz, seed, run)
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, taui=10 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-60 * mV, we=0.8 * mV,
              wi=-2 * mV)
    P = NeuronGroup(N, '''dv/dt = (ge+gi-(v-El))/taum : volt
                          dge/dt = -ge/taue : volt
                          dgi/dt = -gi/taui : volt
                          scale : 1''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    P.scale = 'rand()'
    H = PoissonGroup(60, rates=25 * Hz)
    S = Synapses(P, P, on_pre='ge += we', namespace=ns)
    S.connect(p=0.05)
    S.delay = 'rand() * 3*ms'
    T = Synapses(H, P, on_pre='gi += wi', namespace=ns)
    T.connect(p=0.1)
    in_ge = PoissonInput(P, 'ge', 200, 5 * Hz, weight=1 * mV)                               # N*p = 0.1
    in_v = PoissonInput(P[50:250], 'v', 20, 50 * Hz, weight='0.4*mV*(1 + scale)')           # N*p = 0.1
    in_gi = PoissonInput(P[300:400], 'gi', 5, 8000 * Hz, weight=-0.01 * mV)                 # p = 0.8
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    st = StateMonitor(P, 'v', record=[0, 60, 320])
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, state=st)


def noise_inputs(N=300, duration_ms=200.0, seed_value=303):
    """randn() in the step loop: a stochastic population (two noise terms per
    neuron, Euler-Maruyama) and a second noisy group of odd size, so randn()'s
    kept value passes from site to site and from step to step (one is kept
    already where the run starts: the second group's initial values draw an
    odd number); a PoissonInput large enough for Brian's normal approximation
    ((float)(randn()*scale + loc)) and one small enough for inversion."""
    from brian2 import (NeuronGroup, PoissonInput, Synapses, SpikeMonitor, PopulationRateMonitor, StateMonitor,
                        ms, mV, Hz, seed, run)
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-60 * mV, sigma=3 * mV, sig_e=0.5 * mV,
              we=0.5 * mV, wq=1 * mV)
    P = NeuronGroup(N, '''dv/dt = (ge - (v - El))/taum + sigma*xi*taum**-0.5 : volt
                          dge/dt = -ge/taue + sig_e*xi_e*taue**-0.5 : volt''',
                    threshold='v>Vt', reset='v = Vr', method='euler', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    Q = NeuronGroup(51, 'dx/dt = -x/(10*ms) + 0.5*xi/sqrt(ms) : 1', threshold='x > 0.8', reset='x = 0',
                    method='euler', namespace=ns)
    Q.x = 'randn() * 0.1'
    S = Synapses(P, P, on_pre='ge += we', namespace=ns)
    S.connect(p=0.05)
    S.delay = 'rand() * 2*ms'
    T = Synapses(Q, P, on_pre='ge += wq', namespace=ns)
    T.connect(p=0.1)
    in_big = PoissonInput(P, 'ge', 5000, 20 * Hz, weight=0.05 * mV)         # N*p = 10: normal approximation
    in_small = PoissonInput(P[0:100], 'v', 50, 40 * Hz, weight=0.3 * mV)    # N*p = 0.2: inversion
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    q_mon = SpikeMonitor(Q)
    st = StateMonitor(P, 'v', record=[0, 150, 299])
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, state=st, other_spikes=q_mon)


def regular_ops(N=200, duration_ms=200.0, seed_value=404):
    """Operations (run_regularly): a drive current rewritten every 10 steps
    from t and the neuron index (start slot, before the state monitor), a kick
    to a subgroup every 20 steps, and a decay of ge in the end slot of every
    step (after the reset); recurrent synapses with delays; a state monitor on
    a clock of 5 steps."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, StateMonitor, ms, mV, seed,
                        run)
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-60 * mV, we=0.6 * mV, I0=8 * mV)
    P = NeuronGroup(N, '''dv/dt = (I + ge - (v - El))/taum : volt
                          dge/dt = -ge/taue : volt
                          I : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    P.run_regularly('I = I0 * (1 + (t/ms % 20)/20) * (1 + 0.002*i)', dt=1 * ms)
    P[50:150].run_regularly('v = v + 0.5*mV', dt=2 * ms)
    P.run_regularly('ge = ge * 0.9', when='end')
    S = Synapses(P, P, on_pre='ge += we', namespace=ns)
    S.connect(p=0.05)
    S.delay = 'rand() * 2*ms'
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    st = StateMonitor(P, 'v', record=[0, 60, 199], dt=0.5 * ms)
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, state=st)


def end_monitor(N=300, duration_ms=150.0, seed_value=505):
    """A state monitor in the end slot (after the resets and an end-slot
    operation): refractory LIF neurons with an adaptation current, recurrent
    synapses with delays."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, StateMonitor, ms, mV, seed,
                        run)
    seed(seed_value)
    ns = dict(taum=20 * ms, tauw=50 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-49 * mV, we=0.4 * mV, b=1 * mV)
    P = NeuronGroup(N, '''dv/dt = (El - v - w)/taum : volt (unless refractory)
                          dw/dt = -w/tauw : volt''',
                    threshold='v>Vt', reset='v = Vr; w += b', refractory=3 * ms, method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    P.run_regularly('w = w * 0.999', when='end')
    S = Synapses(P, P, on_pre='v += we', namespace=ns)
    S.connect(p=0.05)
    S.delay = 'rand() * 2*ms'
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    st = StateMonitor(P, 'v', record=[0, 100, 299], when='end')
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, state=st)


def host_sets(N=200, seed_value=606):
    """Three runs with assignments between them and after the last: a drive
    current set for the whole group, a slice of membrane potentials, one
    neuron's current (the reference's set_by_constant, set_array_by_array,
    set_by_single_value); recurrent synapses with delays (spikes in flight
    across the runs).  Runs with build_on_run=False and an explicit build."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, StateMonitor, ms, mV, seed,
                        run)
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-60 * mV, we=0.5 * mV)
    P = NeuronGroup(N, '''dv/dt = (I + ge - (v - El))/taum : volt
                          dge/dt = -ge/taue : volt
                          I : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    P.I = 8 * mV
    S = Synapses(P, P, on_pre='ge += we', namespace=ns)
    S.connect(p=0.05)
    S.delay = 'rand() * 2*ms'
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    st = StateMonitor(P, 'v', record=[0, 5, 150])
    run(50 * ms)
    P.I = 12 * mV
    P.v[:10] = -55 * mV
    run(50 * ms)
    P.I[5] = 0 * mV
    run(50 * ms)
    P.I = 3 * mV
    return dict(P=P, spikes=s_mon, rate=r_mon, state=st)


host_sets.multiple_runs = True


def spike_vars(N=400, duration_ms=200.0, seed_value=707):
    """Spike monitors recording variables (``monitors/spikemonitor.py:62-67``):
    the whole group with v and ge, a subgroup with gi and lastspike.  Every
    pathway has a delay, and one of them writes v itself, so the values must
    be those the thresholder saw (after the update, before the step's
    deliveries and its reset; lastspike already set to the spike's time)."""
    from brian2 import NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, ms, mV, seed, run
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, taui=10 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-49 * mV,
              we=1.62 * mV, wi=-9 * mV, wv=0.5 * mV)
    P = NeuronGroup(N, '''dv/dt  = (ge+gi-(v-El))/taum : volt (unless refractory)
                          dge/dt = -ge/taue : volt
                          dgi/dt = -gi/taui : volt''',
                    threshold='v>Vt', reset='v = Vr', refractory=2 * ms, method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    Ne = int(0.8 * N)
    Ce = Synapses(P[:Ne], P, on_pre='ge += we', delay=0.1 * ms, namespace=ns)
    Ci = Synapses(P[Ne:], P, on_pre='gi += wi', delay=0.1 * ms, namespace=ns)
    Cv = Synapses(P, P, on_pre='v += wv', delay=0.3 * ms, namespace=ns)
    Ce.connect(p=0.02)
    Ci.connect(p=0.02)
    Cv.connect(p=0.02)
    s_mon = SpikeMonitor(P, variables=['v', 'ge'])
    sub_mon = SpikeMonitor(P[100:300], variables=['gi', 'lastspike'])
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, other_spikes=sub_mon, spike_var_monitors=[s_mon, sub_mon])


def custom_events(N=300, duration_ms=200.0, seed_value=808):
    """A custom event (``NeuronGroup(events=...)``, ``groups/neurongroup.py:522-560``):
    'high' while the potential is above -52 mV.  Its ``run_on_event`` code
    changes v as the spike reset does (the two resets run in the schedule's
    order, before the next update) and drives an adaptation current; a pathway
    ``on_event='high'`` with a delay, and an ``EventMonitor`` recording v."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, EventMonitor, PopulationRateMonitor, ms, mV, seed,
                        run)
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, taua=50 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-49 * mV, Vh=-52 * mV,
              we=0.8 * mV, wh=0.3 * mV, da=0.001 * mV, dvh=0.0005 * mV)
    P = NeuronGroup(N, '''dv/dt = (ge - gh - a - (v - El))/taum : volt
                          dge/dt = -ge/taue : volt
                          dgh/dt = -gh/taue : volt
                          da/dt = -a/taua : volt''',
                    threshold='v>Vt', reset='v = Vr', events={'high': 'v > Vh'}, method='exact', namespace=ns)
    P.run_on_event('high', 'a += da; v -= dvh')
    P.v = 'Vr + rand() * (Vt - Vr)'
    S = Synapses(P, P, on_pre='ge += we', delay=0.2 * ms, namespace=ns)
    S.connect(p=0.05)
    Sh = Synapses(P, P, on_pre='gh += wh', on_event='high', delay=0.5 * ms, namespace=ns)
    Sh.connect(p=0.02)
    s_mon = SpikeMonitor(P)
    e_mon = EventMonitor(P, 'high', variables=['v'])
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, other_spikes=e_mon, spike_var_monitors=[e_mon])


def synaptic_state(N=300, duration_ms=150.0, seed_value=909):
    """Per-synapse state of a Synapses object: a clock-driven trace x
    (``synapses/synapses.py:779-794``, the groups slot) that on_pre also
    raises, ``run_regularly`` code on the synapses every 1 ms changing the
    weights from the trace, and state monitors of synaptic variables (start
    slot, several synapses; end slot, one)."""
    from brian2 import (NeuronGroup, Synapses, SpikeMonitor, PopulationRateMonitor, StateMonitor, ms, mV, seed,
                        run)
    seed(seed_value)
    ns = dict(taum=20 * ms, taue=5 * ms, taux=15 * ms, Vt=-50 * mV, Vr=-60 * mV, El=-49 * mV, we=0.6 * mV,
              dw=0.02 * mV, wmax=1.5 * mV)
    P = NeuronGroup(N, '''dv/dt = (ge - (v - El))/taum : volt
                          dge/dt = -ge/taue : volt''',
                    threshold='v>Vt', reset='v = Vr', method='exact', namespace=ns)
    P.v = 'Vr + rand() * (Vt - Vr)'
    S = Synapses(P, P, '''w : volt
                          dx/dt = -x/taux : 1 (clock-driven)''',
                 on_pre='ge += w; x += 1', delay=0.2 * ms, namespace=ns)
    S.connect(p=0.05)
    S.w = 'we * (0.5 + rand())'
    S.run_regularly('w = clip(w + dw * (x - 0.5), 0*mV, wmax)', dt=1 * ms)
    st = StateMonitor(S, ['w', 'x'], record=[0, 7, 42, 100])
    st_end = StateMonitor(S, 'w', record=[3], when='end')
    s_mon = SpikeMonitor(P)
    r_mon = PopulationRateMonitor(P)
    run(duration_ms * ms)
    return dict(P=P, spikes=s_mon, rate=r_mon, S=S, syn_vars=['w', 'x'], syn_state=[st, st_end])

SCENARIOS = {
    "lif_refractory": lif_refractory,
    "hetero_delays": hetero_delays,
    "subgroup_monitors": subgroup_monitors,
    "input_group": input_group,
    "presynaptic_read": presynaptic_read,
    "spike_generator": spike_generator,
    "stdp": stdp,
    "gap_junctions": gap_junctions,
    "explicit_methods": explicit_methods,
    "poisson_input": poisson_input,
    "poisson_drive": poisson_drive,
    "noise_inputs": noise_inputs,
    "regular_ops": regular_ops,
    "end_monitor": end_monitor,
    "host_sets": host_sets,
    "spike_vars": spike_vars,
    "custom_events": custom_events,
    "synaptic_state": synaptic_state,
}


# ---------------------------------------------------------------------------
# The adjoint benchmark's network ("adjoint gradients" configuration) as a
# Brian script: the forward pass the reference computes for it (on_pre
# delivery at the step grid).  Inputs, weights, initial state come from
# brian2_gb300.adjoint.make_problem (seeded numpy).
# ---------------------------------------------------------------------------
def adjoint_network(seed=42, steps=5000, n_in=200, n_h=1000, n_o=10):
    """200 input trains (SpikeGeneratorGroup) -> 1000 exact-linear LIF neurons
    with an exponential current (taum 20 ms, taus 5 ms, CUBA threshold and
    reset) through the dense W, -> 10 non-spiking readout neurons of the same
    dynamics through the dense W_out.  Records the hidden spikes and the
    readout potentials at the end of every step (after the deliveries)."""
    import numpy as np
    from brian2 import (NeuronGroup, Synapses, SpikeGeneratorGroup, SpikeMonitor, StateMonitor,
                        volt, second, run)
    from brian2_gb300.adjoint import AdjointConfig, make_problem
    cfg = AdjointConfig(n_in=n_in, n_h=n_h, n_o=n_o, steps=steps, seed=seed)
    prob = make_problem(cfg)
    ptr, ids = prob["in_ptr"], prob["in_ids"]
    in_steps = np.repeat(np.arange(cfg.steps), np.diff(ptr))
    ns = dict(El=cfg.El * volt, Vt=cfg.Vt * volt, Vr=cfg.Vr * volt, taum=cfg.taum * second, taus=cfg.taus * second)
    eqs = '''
    dv/dt = (El - v + I)/taum : volt
    dI/dt = -I/taus : volt
    '''
    inp = SpikeGeneratorGroup(cfg.n_in, ids, in_steps * cfg.dt * second)
    H = NeuronGroup(cfg.n_h, eqs, threshold='v > Vt', reset='v = Vr', method='exact', namespace=ns)
    O = NeuronGroup(cfg.n_o, eqs, method='exact', namespace=ns)
    s0 = prob["state0"]
    H.v = s0[:cfg.n_h] * volt
    O.v = s0[2 * cfg.n_h:2 * cfg.n_h + cfg.n_o] * volt
    Sin = Synapses(inp, H, 'w : volt', on_pre='I_post += w')
    ii, jj = np.meshgrid(np.arange(cfg.n_in), np.arange(cfg.n_h), indexing="ij")
    Sin.connect(i=ii.ravel(), j=jj.ravel())
    Sin.w = prob["W"].ravel() * volt
    Sout = Synapses(H, O, 'w : volt', on_pre='I_post += w')
    hh, oo = np.meshgrid(np.arange(cfg.n_h), np.arange(cfg.n_o), indexing="ij")
    Sout.connect(i=hh.ravel(), j=oo.ravel())
    Sout.w = prob["W_out"].ravel() * volt
    spikes = SpikeMonitor(H)
    readout = StateMonitor(O, 'v', record=True, when='end')
    run(cfg.steps * cfg.dt * second)
    return dict(P=H, O=O, Sin=Sin, Sout=Sout, spikes=spikes, readout=readout)
