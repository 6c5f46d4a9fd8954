"""The model program's time loop (ccsm.F90:40-63) around the GPU step: output
times, step counts and the MCR/ECR records."""
import pytest

from conformal_cubed_sphere_gb300 import driver as D


def test_default_time_settings_follow_the_namelist_defaults():
    ts = D.TimeSettings()
    assert (ts.dt, ts.total_run_time, ts.nsteps, ts.history_interval) == (300.0, 86400, 288, 360)
    assert ts.total_output_num == 240
    # mod(it*300, 360) == 0 only every sixth step: 48 outputs, the last at the end
    steps = D.output_steps(ts)
    assert steps == list(range(6, 289, 6))


def test_output_times_in_double_precision():
    ts = D.TimeSettings(dt=600.0, run_days=0, run_hours=6, history_interval=3600)
    assert ts.nsteps == 36 and D.output_steps(ts) == [6, 12, 18, 24, 30, 36]
    # a dt that never lands on the interval writes nothing, as the reference would
    ts = D.TimeSettings(dt=7.3, run_days=0, run_hours=1, history_interval=600)
    assert ts.nsteps == int(3600 / 7.3)
    assert D.output_steps(ts) == [it for it in range(1, ts.nsteps + 1) if (it * 7.3) % 600.0 == 0.0]


def test_truncating_step_count():
    ts = D.TimeSettings(dt=700.0, run_days=0, run_hours=1)
    assert ts.nsteps == 5  # 3600 / 700 = 5.14 -> 5


class _FakeStepper:
    """Counts steps; diag returns (mass, energy) as functions of the step count."""

    def __init__(self):
        self.n = 0
        self.calls = []

    def step(self, k):
        assert k >= 1
        self.n += k
        self.calls.append(k)

    def diag(self):
        return 100.0 + self.n, 1000.0 + 2 * self.n

    def get_state(self):
        return self.n

    def check_state(self):
        return 0 if self.n < 1000 else 7


def test_run_chunks_steps_and_uses_old_state_energy():
    ts = D.TimeSettings(dt=600.0, run_days=0, run_hours=2, history_interval=1800)
    f = _FakeStepper()
    seen = []
    recs = D.run(f, ts, on_output=lambda idx, st: seen.append((idx, st)), log=None)
    assert f.n == ts.nsteps == 12
    assert [r.step for r in recs] == [3, 6, 9, 12]
    assert seen == [(1, 0), (2, 3), (3, 6), (4, 9), (5, 12)]
    # mass of the output state, energy of the state one step earlier
    assert recs[0].mcr == pytest.approx(3 / 100.0)
    assert recs[0].ecr == pytest.approx(2 * 2 / 1000.0)
    g = _FakeStepper()
    recs = D.run(g, ts, energy_of_new_state=True, log=None)
    assert recs[0].ecr == pytest.approx(2 * 3 / 1000.0)
    assert g.calls == [3, 3, 3, 3]


def test_unknown_scheme_rejected():
    with pytest.raises(ValueError):
        D.run(_FakeStepper(), D.TimeSettings(integral_scheme="Euler"), log=None)


@pytest.mark.gpu
def test_driver_on_the_gpu_matches_stepping_by_hand():
    import numpy as np

    from conformal_cubed_sphere_gb300 import model as M
    from tests.helpers import seeded_case

    mesh, s, dt = seeded_case(12, 3, oro=True)
    dt = float(int(dt))  # whole seconds, as namelist settings are
    ts = D.TimeSettings(dt=dt, run_days=0, run_hours=0, run_minutes=0, run_seconds=int(12 * dt),
                        history_interval=int(4 * dt))
    a = M.Stepper(mesh, dt, precision="fp64")
    a.set_state(s)
    states = {}
    recs = D.run(a, ts, on_output=lambda idx, st: states.__setitem__(idx, st), log=None)
    b = M.Stepper(mesh, dt, precision="fp64")
    b.set_state(s)
    m0, e0 = b.diag()
    for r in recs:
        b.step(r.step - 1 - (0 if r.output_idx == 2 else recs[r.output_idx - 3].step))
        e_old = b.diag()[1]
        b.step(1)
        m_new = b.diag()[0]
        assert r.mcr == (m_new - m0) / m0 and r.ecr == (e_old - e0) / e0
        got = b.get_state()
        for k in ("phiG", "u", "v"):
            assert np.array_equal(states[r.output_idx][k], got[k])


def _driver_binary():
    from conformal_cubed_sphere_gb300 import build as B
    B.build()
    return str(B.DRIVER)


def test_cpp_driver_plan_matches_the_python_time_loop():
    """The C++ model program over the C ABI computes the same step count and output
    steps as the Python loop (--plan: host work only, no GPU)."""
    import subprocess

    r = subprocess.run([_driver_binary(), "--N", "12", "--plan", "--run-days", "0", "--run-hours", "6", "--dt",
                        "600", "--history-interval", "3600"], capture_output=True, text=True, check=True)
    steps = [int(l.split()[-1]) for l in r.stdout.splitlines() if l.startswith(" output step")]
    ts = D.TimeSettings(dt=600.0, run_days=0, run_hours=6, history_interval=3600)
    assert steps == D.output_steps(ts)
    assert f"nsteps {ts.nsteps} " in r.stdout


@pytest.mark.gpu
def test_cpp_driver_matches_the_python_api(tmp_path):
    """The C++ driver (mesh, initial state, time loop, all through the C ABI) ends in
    the same FP64 state as the Python binding stepping the same case."""
    import subprocess

    import numpy as np

    from conformal_cubed_sphere_gb300 import _lib as L
    from conformal_cubed_sphere_gb300 import model as M

    mesh = M.Mesh(16, 3)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=3, lmax_oro=8)
    dt = float(int(M.cfl_dt(mesh, s, 0.5)))
    out = tmp_path / "final.bin"
    r = subprocess.run([_driver_binary(), "--N", "16", "--precision", "fp64", "--case", "seeded", "--seed", "3",
                        "--lmax-oro", "8", "--radius", str(mesh.radius), "--dt", repr(dt), "--run-days", "0",
                        "--run-seconds", str(int(12 * dt)), "--history-interval", str(int(4 * dt)), "--out",
                        str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if "MCR, ECR" in l]
    assert len(lines) == 4  # the initial line and three outputs
    g = M.Stepper(mesh, dt, precision="fp64")
    g.set_state(s)
    g.step(12)
    ref = g.get_state()
    got = np.fromfile(out, dtype=np.float64).reshape(3, mesh.ncell)
    m = ~mesh.corner_mask()
    for k, name in enumerate(("phiG", "u", "v")):
        assert np.array_equal(got[k][m].view(np.int64), ref[name][m].view(np.int64)), name


def test_cpp_driver_reads_a_mesh_file(tmp_path):
    """--mesh-file: the driver takes N from the raw-binary mesh file (host only, --plan)."""
    import subprocess

    from conformal_cubed_sphere_gb300 import model as M

    path = tmp_path / "c10.ccsmesh"
    M.Mesh(10, 3).save(path)
    r = subprocess.run([_driver_binary(), "--mesh-file", str(path), "--plan", "--run-days", "0", "--run-hours",
                        "1", "--dt", "600", "--history-interval", "1800"], capture_output=True, text=True,
                       check=True)
    assert " N 10 halo 3 dt 600 nsteps 6 outputs 2" in r.stdout
    bad = subprocess.run([_driver_binary(), "--mesh-file", str(tmp_path / "absent"), "--plan"],
                         capture_output=True, text=True)
    assert bad.returncode != 0 and "mesh file" in bad.stderr


def test_run_stops_on_a_bad_state():
    class Blowup(_FakeStepper):
        def check_state(self):
            return 3 if self.n >= 6 else 0

    ts = D.TimeSettings(dt=600.0, run_days=0, run_hours=2, history_interval=1800)
    with pytest.raises(FloatingPointError, match="step 6: 3 cells"):
        D.run(Blowup(), ts, log=None)
    assert len(D.run(Blowup(), ts, log=None, check=False)) == 4


def test_run_records_and_bounds_the_courant_number():
    class Growing(_FakeStepper):
        def courant(self):
            return 0.1 * self.n

    ts = D.TimeSettings(dt=600.0, run_days=0, run_hours=2, history_interval=1800)
    recs = D.run(Growing(), ts, log=None, max_courant=5.0)
    assert [r.courant for r in recs] == pytest.approx([0.3, 0.6, 0.9, 1.2])
    assert all(r.courant is None for r in D.run(Growing(), ts, log=None))
    with pytest.raises(FloatingPointError, match="step 9: Courant number 0.9 above 0.8"):
        D.run(Growing(), ts, log=None, max_courant=0.8)


@pytest.mark.gpu
def test_cpp_driver_stops_above_the_courant_bound():
    """--max-courant: the C++ driver stops at the first output whose state's Courant
    number exceeds the bound, and runs through below it."""
    import subprocess

    from conformal_cubed_sphere_gb300 import _lib as L
    from conformal_cubed_sphere_gb300 import model as M

    mesh = M.Mesh(12, 3)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=1)
    dt = float(int(M.cfl_dt(mesh, s, 0.5)))  # whole seconds: the outputs land on the interval
    args = [_driver_binary(), "--N", "12", "--precision", "mixed", "--case", "seeded", "--radius",
            str(mesh.radius), "--dt", repr(dt), "--run-days", "0", "--run-seconds", str(int(8 * dt)),
            "--history-interval", str(int(4 * dt))]
    ok = subprocess.run(args + ["--max-courant", "5"], capture_output=True, text=True, timeout=600)
    assert ok.returncode == 0, ok.stderr
    bad = subprocess.run(args + ["--max-courant", "0.01"], capture_output=True, text=True, timeout=600)
    assert bad.returncode == 1 and "Courant number" in bad.stderr


_NAMELIST = """! settings of one run
&time_settings
Run_Days         = 0,
run_hours        = 6
run_minutes      = 0
run_seconds      = 0
dt               = 6.0d2     ! seconds
history_interval = 3600
integral_scheme  = 'RK3_TVD' ! 'RK3_TVD' or 'RK4', a '/' in a comment
/

&case_select
case_num    = 6,
/

&domain
mesh_file   = 'no/such/mesh!file'
xhalo       = 4,  yhalo = 4,
/

&dynamic_opt
reconstruct_scheme = "WENO"
/
"""


def test_namelist_reader(tmp_path):
    path = tmp_path / "namelist.input"
    path.write_text(_NAMELIST)
    nml = D.read_namelist(path)
    assert nml["time_settings"]["run_days"] == 0 and nml["time_settings"]["dt"] == 600.0
    assert nml["time_settings"]["integral_scheme"] == "RK3_TVD"
    assert nml["domain"] == {"mesh_file": "no/such/mesh!file", "xhalo": 4, "yhalo": 4}
    rs = D.settings_from_namelist(path)
    assert rs.time == D.TimeSettings(dt=600.0, run_days=0, run_hours=6, history_interval=3600,
                                     integral_scheme="RK3_TVD")
    assert (rs.case_num, rs.mesh_file, rs.halo, rs.reconstruct_scheme) == (6, "no/such/mesh!file", 4, "WENO")
    # an empty file gives the defaults of parameters_mod.F90:118-128
    empty = tmp_path / "empty.input"
    empty.write_text("")
    assert D.settings_from_namelist(empty).time == D.TimeSettings()
    # value lists and logicals
    other = tmp_path / "other.input"
    other.write_text("&g\n a = 1, 2, 3\n flag = .true.\n s = 'it''s'\n/\n")
    assert D.read_namelist(other)["g"] == {"a": [1, 2, 3], "flag": True, "s": "it's"}


def test_mesh_namelist_resolution(tmp_path):
    path = tmp_path / "mesh.input"
    path.write_text("&domain\n dx = 0.5,\n dy = 0.5,\n gen_method = 'Rancic'\n/\n")
    assert D.mesh_resolution_from_namelist(path) == 180
    path.write_text("&domain\n dx = 0.7\n/\n")
    with pytest.raises(ValueError):
        D.mesh_resolution_from_namelist(path)


def test_cpp_driver_reads_the_namelists(tmp_path):
    """ccsm_gpu --namelist / --mesh-namelist (host only, --plan): the same time
    settings, scheme, halo and resolution as the Python reader."""
    import subprocess

    nl = tmp_path / "namelist.input"
    nl.write_text(_NAMELIST)
    ml = tmp_path / "mesh.input"
    ml.write_text("&domain\n dx = 7.5,\n dy = 7.5\n/\n")
    r = subprocess.run([_driver_binary(), "--namelist", str(nl), "--mesh-namelist", str(ml), "--plan"],
                       capture_output=True, text=True, check=True)
    rs = D.settings_from_namelist(nl)
    steps = [int(l.split()[-1]) for l in r.stdout.splitlines() if l.startswith(" output step")]
    assert steps == D.output_steps(rs.time)
    assert f" N 12 halo 4 dt 600 nsteps {rs.time.nsteps} " in r.stdout
    assert "mesh_file 'no/such/mesh!file' not found" in r.stderr


@pytest.mark.gpu
def test_cpp_driver_runs_a_namelist_case_like_the_python_driver(tmp_path):
    """A run set up only by namelist files (test case 6, RK3_TVD, halo 4, C12 from
    dx = 7.5): the C++ driver's MCR/ECR lines equal the Python driver's records on
    the same case bit for bit (FP64 lane)."""
    import subprocess

    from conformal_cubed_sphere_gb300 import _lib as L
    from conformal_cubed_sphere_gb300 import model as M

    nl = tmp_path / "namelist.input"
    nl.write_text(_NAMELIST)
    ml = tmp_path / "mesh.input"
    ml.write_text("&domain\n dx = 7.5,\n dy = 7.5\n/\n")
    r = subprocess.run([_driver_binary(), "--namelist", str(nl), "--mesh-namelist", str(ml), "--precision", "fp64"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    got = [tuple(float(x) for x in l.split()[-2:]) for l in r.stdout.splitlines() if "MCR, ECR" in l][1:]
    rs = D.settings_from_namelist(nl)
    mesh = M.Mesh(D.mesh_resolution_from_namelist(ml), rs.halo, radius=6371229.0)
    s = M.initial_state(mesh, kind={2: L.CCS_IC_CASE2, 5: L.CCS_IC_CASE5, 6: L.CCS_IC_CASE6}[rs.case_num])
    g = M.Stepper(mesh, rs.time.dt, precision="fp64", scheme=rs.time.integral_scheme)
    g.set_state(s)
    recs = D.run(g, rs.time, log=None)
    assert got == [(rec.mcr, rec.ecr) for rec in recs]


@pytest.mark.gpu
def test_cpp_driver_history_files(tmp_path):
    """--history: one checkpoint file per history time (the initial state included),
    each equal to the Python driver's output state at that time."""
    import subprocess

    import numpy as np

    from conformal_cubed_sphere_gb300 import _lib as L
    from conformal_cubed_sphere_gb300 import model as M

    nl = tmp_path / "namelist.input"
    nl.write_text(_NAMELIST)
    ml = tmp_path / "mesh.input"
    ml.write_text("&domain\n dx = 7.5\n/\n")
    prefix = tmp_path / "hist"
    r = subprocess.run([_driver_binary(), "--namelist", str(nl), "--mesh-namelist", str(ml), "--precision", "fp64",
                        "--history", str(prefix)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rs = D.settings_from_namelist(nl)
    mesh = M.Mesh(12, rs.halo, radius=6371229.0)
    s = M.initial_state(mesh, kind=L.CCS_IC_CASE6)
    g = M.Stepper(mesh, rs.time.dt, precision="fp64", scheme=rs.time.integral_scheme)
    g.set_state(s)
    states = {}
    D.run(g, rs.time, on_output=lambda idx, st: states.__setitem__(idx, st), log=None)
    files = sorted(tmp_path.glob("hist_*.ccsstate"))
    assert [f.name for f in files] == [f"hist_{k:04d}.ccsstate" for k in sorted(states)]
    m = ~mesh.corner_mask()
    for f, k in zip(files, sorted(states)):
        got = M.State.load(f, mesh)
        for name in ("phiG", "u", "v", "phi"):
            assert np.array_equal(got[name][m], states[k][name][m]), (f.name, name)


@pytest.mark.gpu
def test_python_driver_cli_matches_the_cpp_driver(tmp_path):
    """python -m conformal_cubed_sphere_gb300.driver and ccsm_gpu on the same
    namelist files: the same MCR/ECR values and byte-identical history files."""
    import subprocess
    import sys
    from pathlib import Path

    nl = tmp_path / "namelist.input"
    nl.write_text(_NAMELIST)
    ml = tmp_path / "mesh.input"
    ml.write_text("&domain\n dx = 7.5\n/\n")
    common = ["--namelist", str(nl), "--mesh-namelist", str(ml), "--precision", "fp64"]
    c = subprocess.run([_driver_binary()] + common + ["--history", str(tmp_path / "c")], capture_output=True,
                       text=True, timeout=600)
    p = subprocess.run([sys.executable, "-m", "conformal_cubed_sphere_gb300.driver"] + common +
                       ["--history", str(tmp_path / "p")], capture_output=True, text=True, timeout=600,
                       cwd=Path(__file__).resolve().parents[1])
    assert c.returncode == 0, c.stderr
    assert p.returncode == 0, p.stderr + p.stdout

    def values(out):
        return [tuple(float(x) for x in l.split()[-2:]) for l in out.splitlines() if "MCR, ECR" in l]

    assert values(c.stdout) == values(p.stdout) and len(values(p.stdout)) == 7
    cf, pf = sorted(tmp_path.glob("c_*.ccsstate")), sorted(tmp_path.glob("p_*.ccsstate"))
    assert len(cf) == len(pf) == 7
    for a, b in zip(cf, pf):
        assert a.read_bytes() == b.read_bytes(), (a.name, b.name)


def test_python_driver_cli_needs_a_mesh(tmp_path):
    nl = tmp_path / "namelist.input"
    nl.write_text(_NAMELIST)
    with pytest.raises(SystemExit):
        D.main(["--namelist", str(nl)])


def test_a_netcdf_mesh_file_is_not_read_as_raw(tmp_path):
    """The reference's mesh_file is NetCDF: both drivers probe it and generate the
    mesh instead of failing on it; a raw-binary mesh file is recognised."""
    import subprocess

    from conformal_cubed_sphere_gb300 import model as M
    nc = tmp_path / "ccs_mesh.nc"
    nc.write_bytes(b"CDF\x01" + bytes(4096))  # a NetCDF classic header, not a raw-binary mesh
    assert not D.is_raw_mesh_file(nc)
    raw = tmp_path / "mesh.ccsmesh"
    M.Mesh(6, 3).save(raw)
    assert D.is_raw_mesh_file(raw)
    nl = tmp_path / "namelist.input"
    nl.write_text(_NAMELIST.replace("no/such/mesh!file", str(nc)))
    r = subprocess.run([_driver_binary(), "--namelist", str(nl), "--N", "12", "--plan"],
                       capture_output=True, text=True, check=True)
    assert f"mesh_file '{nc}' is not a raw-binary mesh file: the mesh is generated" in r.stderr
    assert " N 12 halo 4 " in r.stdout
