"""Source rules the library relies on, checked on the CPU: every call that
synchronises the whole device goes through the capture gate's wrappers in
utc_gb300/csrc/nb_internal.cuh (nb::dmalloc, nb::dfree, nb::hmalloc,
nb::hfree, nb::dmalloc_managed, nb::device_sync, nb::dmemcpy,
nb::graph_instantiate, nb::graph_exec_destroy), so that no such call can
overlap another thread's step-graph capture, and every capture holds the gate
shared."""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "utc_gb300", "csrc")
DIRECT = re.compile(r"\b(cudaMalloc|cudaMallocHost|cudaMallocManaged|cudaFree|cudaFreeHost|cudaDeviceSynchronize|"
                    r"cudaMemcpy|cudaGraphInstantiate|cudaGraphExecDestroy)\s*\(")


def code_lines(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for k, line in enumerate(text.splitlines(), 1):
        yield k, line.split("//")[0]


def test_device_wide_calls_go_through_the_gate():
    bad = []
    for name in sorted(os.listdir(CSRC)):
        if not name.endswith((".cu", ".cuh")) or name == "nb_internal.cuh":
            continue
        for k, line in code_lines(os.path.join(CSRC, name)):
            if DIRECT.search(line):
                bad.append(f"{name}:{k}: {line.strip()}")
    assert not bad, "\n".join(bad)


def test_every_capture_holds_the_gate():
    for name in sorted(os.listdir(CSRC)):
        if not name.endswith(".cu"):
            continue
        lines = [ln for _, ln in code_lines(os.path.join(CSRC, name))]
        for k, line in enumerate(lines):
            if "cudaStreamBeginCapture(" in line:
                before = "\n".join(lines[max(0, k - 4):k])
                assert "std::shared_lock<std::shared_mutex>" in before and "capture_gate()" in before, \
                    f"{name}:{k + 1}: capture without the gate held shared"
