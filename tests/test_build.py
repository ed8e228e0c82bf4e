"""Every committed spec compiles for sm_103a (nvcc cross-compiles without a GPU)."""
import os
from concurrent.futures import ThreadPoolExecutor

from brian2_gb300 import native, workloads


def test_all_model_libraries_build():
    names = sorted(f[:-5] for f in os.listdir(workloads.SPECS) if f.endswith(".json"))
    with ThreadPoolExecutor(max_workers=8) as ex:
        paths = list(ex.map(lambda n: native.build_model(workloads.load_spec(n)), names))
    assert all(os.path.exists(p) for p in paths)


def test_construction_libraries_build():
    assert os.path.exists(native.build_construct())
    assert os.path.exists(native.build_scale())


def test_push_kernel_keeps_its_registers(tmp_path):
    """The headline's push-mode kernel, in the shapes of up to 512 threads a CTA,
    compiles without register spills: at two CTAs per SM the spills live in the
    L1 that the shared memory leaves, and cost the step measurable time."""
    import re
    import subprocess
    from brian2_gb300.codegen import render_model
    src = tmp_path / "delays_f32.cu"
    src.write_text(render_model(workloads.load_spec("delays_f32")))
    flags = [f for f in native.nvcc_flags(True, True) if f != "-shared"]
    r = subprocess.run([native.nvcc_path()] + flags + ["-Xptxas", "-v", "-c", str(src), "-o", str(tmp_path / "m.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    spills, cur = {}, None
    for ln in r.stderr.splitlines():
        m = re.search(r"Compiling entry function '(\w+)'", ln)
        if m:
            cur = m.group(1)
        m = re.search(r"(\d+) bytes spill stores", ln)
        if m and cur:
            spills[cur] = int(m.group(1))
            cur = None
    push = {k: v for k, v in spills.items() if "b200_push_kernel" in k}
    shapes = {k: v for k, v in push.items() if re.search(r"ILi(256|512)E", k)}
    assert len(shapes) == 3, sorted(push)
    assert all(v == 0 for v in shapes.values()), shapes
