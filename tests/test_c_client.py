"""The C ABI from C: a client compiled with gcc against include/pysit_gb300.h and linked with
libpysit_gb300.so describes a small 2D batch, creates a plan, reads its workspace size, meets
the library's argument checks and destroys the plan; a C++ client makes the library's host
allocations fail and gets a status back.  No GPU call is made (workspace binding and runs need
a device), so this runs on any host with the CUDA runtime library."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CLIENT = r"""
#include <stdio.h>
#include <string.h>
#include "pysit_gb300.h"

int main(void) {
    /* 2 shots on a 30 x 24 grid (4-cell PML each side), order 4, FP32, 50 steps */
    static double prof[4] = {50.0, 35.0, 20.0, 5.0};
    static int64_t sptr[3] = {0, 1, 2}, scell[2] = {100, 200};
    static int32_t spt[2] = {0, 0};
    static double sw[2] = {1.0, 1.0}, amp[2 * 50];
    static int64_t rptr[3] = {0, 2, 4}, rcell[4] = {150, 151, 150, 152};
    static int32_t rpt[4] = {0, 1, 0, 1};
    static double rws[4] = {1, 1, 1, 1}, rwi[4] = {1, 1, 1, 1};
    pysit_plan_desc d;
    pysit_plan* plan = NULL;
    uint64_t bytes = 0;
    int rc;
    memset(&d, 0, sizeof d);
    for (int k = 0; k < 100; ++k) amp[k] = k == 3 ? 1.0 : 0.0;
    d.dim = 2; d.order = 4; d.dtype = PYSIT_F32;
    d.n[0] = 30; d.n[1] = 1; d.n[2] = 24;
    d.delta[0] = d.delta[1] = d.delta[2] = 5.0;
    d.pad_lo[0] = d.pad_hi[0] = d.pad_lo[2] = d.pad_hi[2] = 4;
    d.dt = 1e-4; d.nsteps = 50; d.imaging_period = 1; d.checkpoint_every = 7;
    d.shots_per_launch = 2; d.nshots = 2; d.use_graph = 1;
    for (int a = 0; a < 3; a += 2) {
        d.sig_l[a] = prof; d.nsig_l[a] = 4; d.sig_r[a] = prof; d.nsig_r[a] = 4;
    }
    d.nsrc = 1; d.src_tap_ptr = sptr; d.src_tap_cell = scell; d.src_tap_point = spt;
    d.src_tap_w = sw; d.src_amp = amp;
    d.nrec = 2; d.rec_tap_ptr = rptr; d.rec_tap_cell = rcell; d.rec_tap_point = rpt;
    d.rec_tap_wsample = rws; d.rec_tap_winject = rwi;
    if ((rc = pysit_plan_create(&d, &plan)) != PYSIT_OK) {
        printf("create failed %d: %s\n", rc, pysit_cuda_last_error());
        return 1;
    }
    if (pysit_cuda_version() != PYSIT_ABI_VERSION) return 5;
    if (pysit_plan_workspace_bytes(plan, &bytes) != PYSIT_OK || bytes == 0) return 2;
    /* a run before a workspace is bound is an error, not a crash */
    if (pysit_plan_forward(plan, NULL, NULL) != PYSIT_EINVAL) return 3;
    pysit_plan_destroy(plan);
    /* argument checks */
    d.order = 5;
    if (pysit_plan_create(&d, &plan) != PYSIT_EINVAL) return 4;
    printf("ok %llu %s\n", (unsigned long long)bytes, pysit_cuda_last_error());
    return 0;
}
"""


# A C++ client whose replacement operator new (which the library's own allocations resolve to)
# throws while armed: every entry point must turn the exception into PYSIT_EHOST.
FAILING_NEW = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include "pysit_gb300.h"

static bool g_fail = false;
void* operator new(std::size_t n) {
    if (g_fail) throw std::bad_alloc();
    if (void* p = std::malloc(n ? n : 1)) return p;
    throw std::bad_alloc();
}
void operator delete(void* p) noexcept { std::free(p); }
void operator delete(void* p, std::size_t) noexcept { std::free(p); }

int main() {
    static double prof[4] = {50.0, 35.0, 20.0, 5.0};
    static int64_t sptr[2] = {0, 1}, scell[1] = {100};
    static int32_t spt[1] = {0};
    static double sw[1] = {1.0}, amp[20];
    pysit_plan_desc d;
    std::memset(&d, 0, sizeof d);
    d.dim = 2; d.order = 4; d.dtype = PYSIT_F32;
    d.n[0] = 30; d.n[1] = 1; d.n[2] = 24;
    d.delta[0] = d.delta[1] = d.delta[2] = 5.0;
    d.pad_lo[0] = d.pad_hi[0] = d.pad_lo[2] = d.pad_hi[2] = 4;
    d.dt = 1e-4; d.nsteps = 20; d.imaging_period = 1; d.checkpoint_every = 5;
    d.shots_per_launch = 1; d.nshots = 1; d.use_graph = 1;
    for (int a = 0; a < 3; a += 2) { d.sig_l[a] = prof; d.nsig_l[a] = 4; d.sig_r[a] = prof; d.nsig_r[a] = 4; }
    d.nsrc = 1; d.src_tap_ptr = sptr; d.src_tap_cell = scell; d.src_tap_point = spt;
    d.src_tap_w = sw; d.src_amp = amp;
    pysit_plan* plan = nullptr;
    g_fail = true;
    int rc = pysit_plan_create(&d, &plan);
    g_fail = false;
    if (rc != PYSIT_EHOST || plan) { std::printf("create: %d\n", rc); return 1; }
    std::printf("%s\n", pysit_cuda_last_error());
    pysit_group* grp = nullptr;
    if (pysit_plan_create(&d, &plan) != PYSIT_OK) return 2;
    g_fail = true;
    rc = pysit_group_create(&plan, 1, &grp);
    g_fail = false;
    if (rc != PYSIT_EHOST || grp) { std::printf("group: %d\n", rc); return 3; }
    std::printf("%s\n", pysit_cuda_last_error());
    pysit_plan_destroy(plan);
    std::printf("ok\n");
    return 0;
}
"""


def _compile_and_run(tmp_path, compiler, name, source, flags):
    from pysit_gb300 import build
    lib = build.build()
    if not shutil.which(compiler):
        pytest.skip(f"{compiler} absent")
    src = tmp_path / name
    src.write_text(source)
    exe = tmp_path / "client"
    libdir = os.path.dirname(lib)
    cmd = [compiler, *flags, "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-lpysit_gb300", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    env = dict(os.environ)
    cuda_lib = "/usr/local/cuda/lib64"
    env["LD_LIBRARY_PATH"] = os.pathsep.join(p for p in (libdir, cuda_lib, env.get("LD_LIBRARY_PATH", "")) if p)
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_c_client_creates_and_destroys_a_plan(tmp_path):
    out = _compile_and_run(tmp_path, "gcc", "client.c", CLIENT, ["-std=c11"])
    assert out.startswith("ok ")
    assert "order" in out


def test_host_allocation_failure_returns_a_status(tmp_path):
    """No C++ exception crosses the C ABI: a failed host allocation inside pysit_plan_create or
    pysit_group_create returns PYSIT_EHOST with a message, and the library stays usable."""
    out = _compile_and_run(tmp_path, "g++", "client.cpp", FAILING_NEW, ["-std=c++17"]).splitlines()
    assert out[0] == "pysit_plan_create: host memory allocation failed"
    assert out[1] == "pysit_group_create: host memory allocation failed"
    assert out[-1] == "ok"
