"""The reference's own standalone-compatible tests through the set_device('b200')
plugin, with the oracle standing in for the GPU (CPU only; not collected by
pytest).  The device registered here as 'b200_oracle' is the plugin's device
with one change: the job it writes runs on the oracle (test infrastructure)
instead of the CUDA library; its outputs are imported the same way.  Brian's
test runner (brian2/tests/__init__.py:142-431) sets the device for every test
marked standalone_compatible, so each selected test builds the reference's
standalone project, runs its construction, records the run through the plugin
and checks the results the plugin writes back -- the reference's known-answer
tests applied to the plugin's translation of the step loop.  Tests that use
features the plugin refuses raise NotImplementedError and count as skipped.

    bash oracle/make_ref_env.sh
    PYTHONPATH=oracle/_ref/pyenv python tests/reference_suite.py [-k EXPRESSION]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from brian2.devices.device import all_devices  # noqa: E402

from brian2_gb300.brian_device import B200Device  # noqa: E402
from oracle import run_job_on_oracle  # noqa: E402


class B200OracleDevice(B200Device):
    """The plugin's device, its jobs run on the oracle."""

    def _run_on_gpu(self):
        directory = self.b200_export_job(os.path.join(self.project_dir, "b200_job"))
        out = run_job_on_oracle(directory)
        with open(os.path.join(directory, "job.json")) as f:
            job = json.load(f)
        init = np.load(os.path.join(directory, "init.npz"))
        out["ts0"] = np.int64(int(init["ts0"]))
        out["ts_end"] = np.int64(int(init["ts0"]) + sum(int(n) for n in job["runs"]))
        out["device_ms"] = np.float64(0.0)
        if job.get("options", {}).get("profile"):
            # (the oracle has no device profile: one cycle per slot, so that the
            # plugin's mapping of the slots to code objects runs; times are 0)
            from brian2_gb300.codegen import profile_slots
            with open(os.path.join(directory, "spec.json")) as f:
                names = [n for n in profile_slots(json.load(f)) if not n.startswith("unused")]
            out["prof_names"] = np.array(names, dtype=str)
            out["prof_cycles"] = np.ones(len(names))
            out["kernel_ms"] = np.float64(0.0)
        np.savez(os.path.join(directory, "out.npz"), **out)
        self.b200_import_results(directory)


def main(argv):
    import brian2
    from brian2.core.preferences import prefs
    dev = B200OracleDevice()
    all_devices["b200_oracle"] = dev
    all_devices["b200_oracle_simple"] = dev
    prefs.devices.cpp_standalone.openmp_threads = 0
    k = argv[argv.index("-k") + 1] if "-k" in argv else \
        "refractory or thresholder or spikequeue or test_monitor or test_synapses or poisson or spikegenerator"
    ok = brian2.test([], test_codegen_independent=False, test_standalone="b200_oracle",
                     fail_for_not_implemented=False, test_in_parallel=[], reset_preferences=False,
                     additional_args=["-q", "-p", "no:cacheprovider", "-k", k, "-rsfE"])
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
