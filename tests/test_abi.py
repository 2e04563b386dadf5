"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, and fails cleanly (no crash, a status code) where no GPU is visible."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def _header_functions():
    with open(os.path.join(ROOT, "include", "ohpic.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ohpic_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_path():
    names = _header_functions()
    for must in ("ohpic_create", "ohpic_scatter", "ohpic_solve", "ohpic_interp", "ohpic_move",
                 "ohpic_push", "ohpic_step", "ohpic_sort", "ohpic_upload_particles",
                 "ohpic_download_particles", "ohpic_diagnostics", "ohpic_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(ohpic):
    L = C.CDLL(ohpic.LIB_PATH)
    names = _header_functions()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding covers exactly the declared functions
    assert sorted(ohpic.SIGNATURES) == names


def test_config_default(ohpic):
    cfg = ohpic.default_config()
    assert cfg.precision == ohpic.FP64
    assert cfg.weights == ohpic.WEIGHTS_REFERENCE
    assert cfg.sort_every == 20 and cfg.track_ids == 1 and cfg.device == 0
    assert cfg.nx == 0 and cfg.nspecies == 0


def test_status_strings(ohpic):
    L = ohpic.lib()
    for code in range(0, 10):
        assert L.ohpic_status_string(code)
    assert L.ohpic_status_string(ohpic.ERR_UNSUPPORTED).decode().startswith("per-particle")


def test_invalid_configs_rejected_before_device(ohpic):
    """Argument checks run before any CUDA call, so they hold on any host."""
    base = dict(n=(8, 8, 8), dt=0.1, b0=(0, 0, 0), qm=[-1.0], q=[-0.1], capacity=[16])
    bad = [
        dict(base, n=(0, 8, 8)),
        dict(base, qm=[0.0]),
        dict(base, capacity=[-1]),
        dict(base, n=(12, 8, 8), tile=(8, 8, 8)),       # tile must divide n
        dict(base, n=(4096, 8, 8), precision=1),         # FP32 cell packing limit
    ]
    for kw in bad:
        cfg = ohpic.make_config(**kw)
        with pytest.raises(ohpic.OhpicError) as e:
            ohpic.PicContext(cfg)
        assert e.value.status == ohpic.ERR_INVALID
    cfg = ohpic.make_config(**base)
    cfg.nspecies = 9
    with pytest.raises(ohpic.OhpicError):
        ohpic.PicContext(cfg)


def test_null_arguments(ohpic):
    L = ohpic.lib()
    assert L.ohpic_create(None, None) == ohpic.ERR_INVALID
    assert L.ohpic_destroy(None) == ohpic.OK
    assert L.ohpic_scatter(None) == ohpic.ERR_INVALID
    assert L.ohpic_step(None, 0.1, 1) == ohpic.ERR_INVALID


_CPP_PROG = r'''
#include <cstdio>
#include "ohpic_modules.hpp"
int main(int argc, char **argv)
{
    ohpic_config cfg;
    ohpic_config_default(&cfg);
    cfg.nx = cfg.ny = cfg.nz = 8;
    cfg.nspecies = 2;
    cfg.precision = OHPIC_FP32;
    cfg.qm[0] = -1.0; cfg.qm[1] = 0.01;
    cfg.q[0] = -0.125; cfg.q[1] = 0.125;
    cfg.capacity[0] = cfg.capacity[1] = 8 * 512;
    cfg.b0[2] = 0.5;
    try {
        ohpic::Context c(cfg);
        ohpic_species_init sp[2] = {};
        for (int s = 0; s < 2; ++s) {
            sp[s].ppc = 4; sp[s].vth = s ? 0.1 : 1.0;
            for (int d = 0; d < 3; ++d) sp[s].hi[d] = 1e30;
        }
        int64_t counts[2];
        c.check(ohpic_init_particles(c.get(), 42, 52, 0, sp, counts), "init");
        ohpic::FieldSolver(c).solve();
        c.step(0.1, 2);
        ohpic::create_particle_mover("boris", c).move_all(0.1);
        ohpic::Scatter(c).scatter_all();
        std::vector<double> e = ohpic::Interpolator(c).interp_all(0, counts[0]);
        ohpic_diag d = c.diagnostics();
        int unsupported = 0, unknown = 0;
        try { double p[6] = {0}; double eb[6] = {0}; ohpic::create_particle_mover("boris", c).move(p, -1.0, eb, 0.1); }
        catch (const ohpic::Error &x) { unsupported = x.status(); }
        try { ohpic::create_particle_mover("leapfrog", c); } catch (const ohpic::Error &x) { unknown = x.status(); }
        // a unit charge at the centre of a 4^3 block with walls on x, mirrors on y, periodic z
        const int32_t nb[3] = {4, 4, 4}, kinds[3] = {OHPIC_BC_DIRICHLET, OHPIC_BC_NEUMANN, OHPIC_BC_PERIODIC};
        const double bv[6] = {0, 0, 0, 0, 0, 0};
        ohpic::BoundedFieldSolver bs(nb, kinds, bv, OHPIC_TABLE_CORRECTED);
        std::vector<double> rho(125, 0.0), phi(125, 0.0);
        rho[2 + 5 * (2 + 5 * 2)] = 1.0;
        bs.solve(rho.data(), phi.data());
        std::printf("ok %lld %lld %zu %d %d %.17g %.17g %.17g\n", (long long)d.count[0], (long long)d.count[1],
                    e.size(), unsupported, unknown, d.total_charge, phi[2 + 5 * (2 + 5 * 2)], phi[0]);
    } catch (const ohpic::Error &x) {
        std::printf("error %d %s\n", x.status(), x.what());
    }
    return 0;
}
'''


def _build_cpp(ohpic, tmp_path):
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    src = tmp_path / "mirror.cpp"
    src.write_text(_CPP_PROG)
    exe = tmp_path / "mirror"
    libdir = os.path.dirname(ohpic.LIB_PATH)
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-lohpic", f"-Wl,-rpath,{libdir}", "-L/usr/local/cuda/lib64",
                        "-Wl,-rpath,/usr/local/cuda/lib64"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout.split()


def test_cpp_mirror_compiles_and_reports_errors(ohpic, tmp_path):
    """The C++ mirror links against the library; without a device the context
    constructor throws ohpic::Error carrying the status code."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible: the GPU test covers this binary")
    words = _build_cpp(ohpic, tmp_path)
    assert words[0] == "error" and int(words[1]) == ohpic.ERR_CUDA


@pytest.mark.gpu
def test_cpp_mirror_runs_the_path(ohpic, tmp_path):
    words = _build_cpp(ohpic, tmp_path)
    assert words[0] == "ok", words
    n0, n1, ne, unsupported, unknown = (int(w) for w in words[1:6])
    assert n0 == n1 == 4 * 512 and ne == 3 * n0
    assert unsupported == ohpic.ERR_UNSUPPORTED and unknown == ohpic.ERR_INVALID
    # FP32 rho: neutral to rounding, relative to the 4 * 512 * 0.125 = 256 charge per species
    assert abs(float(words[6])) < 1e-9 * 256 * 100
    # the bounded solve: a positive potential at the charge, zero on the Dirichlet wall
    assert float(words[7]) > 0.0 and float(words[8]) == 0.0


def test_struct_layouts_match_the_header(ohpic, tmp_path):
    """The ctypes mirrors of the header's structs have the C compiler's sizes and
    field offsets (a field added on one side only would shift the others)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("no gcc")
    from ohhelppic3d_gb300 import serve as S
    pairs = [("ohpic_config", ohpic.Config), ("ohpic_diag", ohpic.Diag),
             ("ohpic_species_init", ohpic.SpeciesInit), ("ohpic_tuning", ohpic.Tuning),
             ("ohpic_serve_config", S.ServeConfig), ("ohpic_run_request", S.RunRequest),
             ("ohpic_run_result", S.RunResult), ("ohpic_serve_stats", S.ServeStats)]
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "ohpic.h"', '#include "ohpic_serve.h"',
             'int main(void) {']
    for cname, py in pairs:
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60).stdout.split("\n")
    got = {tuple(ln.split()[:2]): int(ln.split()[2]) for ln in out if ln.strip()}
    for cname, py in pairs:
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
