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
                wscale=1.0 / 50, dmin_ms=0.1, dmax_ms=5.0):
    """Large CUBA: fixed in-degree K split 80/20 between E and I sources.

    Every neuron receives exactly ``ne_frac*K`` synapses from distinct sources
    drawn uniformly from the excitatory population and ``K - ne_frac*K`` from the
    inhibitory one (``sample(N_pre, size=...)`` per target).  Weights are a
    per-synapse variable ``w`` and delays are drawn uniformly per synapse.
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
    run(duration_ms * ms)
    return dict(P=P, Ce=Ce, Ci=Ci, spikes=s_mon, rate=r_mon)
