"""The boundary's C and C++ side, built and run: the bms2 command-line driver
(the reference driver's flags, BMS2.cpp:7-393 with library/src/utils.hpp:39-87)
and the two code snippets a maintainer copies into the reference's driver
(the C++ facade bms.hpp call for call, and the plain C ABI), each compiled
here against include/ and libbms.so and run on seeded inputs in the
reference's text format.  Their "# Matches", GMCR pair count and candidate
statistics (CandidatesInspector, library/src/utils.hpp:159-178) must equal the
oracle's."""
import json
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from bms2_gb300 import Graphs, build, workloads

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
R = 6


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    t = tmp_path_factory.mktemp("cli")
    q, d = workloads.make("mol1k", 21, n_data=300, n_queries=20)
    q.write_file(t / "queries.txt")
    d.write_file(t / "data.txt")
    qa = Graphs.parse_file(t / "queries.txt").arrays()
    da = Graphs.parse_file(t / "data.txt").arrays()
    return t, qa, da


def cli(*args, cwd=None) -> subprocess.CompletedProcess:
    r = subprocess.run([str(build.CLI), *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=300)
    assert r.returncode == 0, r.stderr
    return r


def field(out: str, name: str) -> int:
    m = re.search(rf"^# {name}: (\d+)$", out, re.M)
    assert m, f"no '# {name}' line in:\n{out}"
    return int(m.group(1))


def test_cli_find_all_and_find_first(inputs):
    t, qa, da = inputs
    want = oracle.run_pipeline(qa, da, R, keep_steps=False)
    r = cli("-Q", t / "queries.txt", "-D", t / "data.txt", "-i", R, "--find-all")
    assert field(r.stdout, "Matches") == want.total > 0
    assert field(r.stdout, "GMCR pairs") == len(want.qidx)
    first = oracle.run_pipeline(qa, da, R, find_first=True, keep_steps=False)
    r = cli("-Q", t / "queries.txt", "-D", t / "data.txt", "-i", R)
    assert field(r.stdout, "Matches") == first.total


def test_cli_reference_semantics_and_json(inputs):
    t, qa, da = inputs
    lit = oracle.run_pipeline(qa, da, R, dfs_literal=True, keep_steps=False)
    r = cli("-Q", t / "queries.txt", "-D", t / "data.txt", "-i", R, "--find-all", "--semantics", "reference")
    assert field(r.stdout, "Matches") == lit.total
    r = cli("-Q", t / "queries.txt", "-D", t / "data.txt", "-i", R, "--find-all", "--json")
    j = json.loads(r.stdout)
    assert j["matches"] == oracle.run_pipeline(qa, da, R, keep_steps=False).total
    assert j["query_graphs"] == 20 and j["data_graphs"] == 300


def test_cli_candidate_statistics(inputs):
    # -p runs the staged pipeline and prints the reference's candidate
    # statistics over the dense matrix after the last refinement step
    t, qa, da = inputs
    want = oracle.run_pipeline(qa, da, R)
    per_node = np.array([int(sum(bin(int(w)).count("1") for w in row)) for row in want.cand])
    r = cli("-Q", t / "queries.txt", "-D", t / "data.txt", "-i", R, "--find-all", "-p")
    assert field(r.stdout, "Total candidates") == int(per_node.sum())
    assert field(r.stdout, "Zero candidates") == int((per_node == 0).sum())
    assert field(r.stdout, "Median candidates") == int(np.sort(per_node)[len(per_node) // 2])
    assert field(r.stdout, "Average candidates") == int(per_node.sum()) // len(per_node)
    assert field(r.stdout, "Matches") == want.total
    printed = [int(x) for x in re.findall(r"^Node \d+: (\d+)$", r.stderr, re.M)]
    assert printed == per_node.tolist()


def test_cli_clustered_join(inputs, tmp_path):
    t, _, da = inputs
    c = workloads.make_cluster_arrays(da, 12, 5, proto_nodes=(3, 5))
    Graphs.from_csr(**c).write_file(tmp_path / "cluster.txt")
    ca = Graphs.parse_file(tmp_path / "cluster.txt").arrays()
    want = oracle.run_pipeline(ca, da, 2, cs=True, keep_steps=False)
    r = cli("-Q", tmp_path / "cluster.txt", "-D", t / "data.txt", "-i", 2, "--find-all", "--use-cs")
    assert field(r.stdout, "Matches") == want.total
    assert field(r.stdout, "Partial matches") == want.n_partial


def snippet(tag: str) -> str:
    text = (ROOT / "INTEGRATION.md").read_text()
    i = text.index(f"tests/test_gpu_cli.py: {tag} -->")
    body = text[i:].split("```", 2)[1]
    return body.split("\n", 1)[1]  # drop the language tag


def compile_and_run(src: str, suffix: str, cwd: Path, *args) -> str:
    compiler = shutil.which("g++" if suffix == ".cpp" else "gcc")
    assert compiler, "no host compiler"
    exe = cwd / f"snippet_{suffix[1:]}"
    (cwd / f"snippet{suffix}").write_text(src)
    std = ["-std=c++17"] if suffix == ".cpp" else ["-std=c11"]
    lib = build.LIB.parent
    r = subprocess.run([compiler, *std, "-O1", "-I", str(ROOT / "include"), str(cwd / f"snippet{suffix}"), "-o",
                        str(exe), "-L", str(lib), "-lbms", f"-Wl,-rpath,{lib}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_integration_cpp_driver_snippet(inputs):
    # the C++ block, with the driver's parsed flags given as `args`
    t, qa, da = inputs
    code = snippet("cpp-driver")
    head = "\n".join(l for l in code.split("\n") if l.startswith("#include") or l.startswith("using namespace"))
    body = "\n".join(l for l in code.split("\n") if not (l.startswith("#include") or l.startswith("using namespace")))
    src = (head + "\n#include <cstdio>\n#include <cstdlib>\n#include <string>\n"
           "struct Args { std::string query_file, data_file; size_t refinement_steps; bool find_all; };\n"
           "int main(int argc, char** argv) {\n"
           "  Args args{argv[1], argv[2], size_t(std::atoi(argv[3])), std::atoi(argv[4]) != 0};\n"
           + body + "\n  std::printf(\"%zu\\n\", total_full_matches);\n  return 0;\n}\n")
    for find_all in (1, 0):
        out = compile_and_run(src, ".cpp", t, t / "queries.txt", t / "data.txt", R, find_all)
        want = oracle.run_pipeline(qa, da, R, find_first=not find_all, keep_steps=False)
        assert int(out.strip()) == want.total


def test_integration_c_abi_snippet(inputs):
    t, qa, da = inputs
    src = ("#include <stdio.h>\n#include <stdlib.h>\n#include \"bms.h\"\nint main(void) {\n" +
           snippet("c-abi").replace('#include "bms.h"', "") +
           "\n  printf(\"%llu\\n\", (unsigned long long)total);\n  return 0;\n}\n")
    out = compile_and_run(src, ".c", t)
    assert int(out.strip()) == oracle.run_pipeline(qa, da, R, keep_steps=False).total
