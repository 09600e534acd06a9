"""pridediff_gb300.dropin: deeprecon's import paths served by this package
(host only; each case runs in a fresh interpreter so sys.modules stays clean)."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(code):
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip()


def test_pridediff_imports_resolve_to_this_package():
    out = _run(
        "import pridediff_gb300.dropin as d; names = d.install(projector=True)\n"
        "from deeprecon.torch.projector import projector2d, projector3d, projectorsp\n"
        "from deeprecon.torch.projector.function import ProjFanFlatDis2d\n"
        "import deeprecon.torch.projector.projector as pm, radontorch\n"
        "import pridediff_gb300 as P\n"
        "assert projector2d is P.projector2d and projectorsp is P.projectorsp\n"
        "assert pm.__name__ == 'pridediff_gb300.projector'\n"
        "assert radontorch is P.radontorch and hasattr(radontorch, 'ProjConeFlatDis3d')\n"
        "assert callable(ProjFanFlatDis2d.apply)\n"
        "print(','.join(names))")
    assert out.split(",")[:2] == ["radontorch", "deeprecon"]


def test_only_the_extension_is_replaced_when_deeprecon_is_installed(tmp_path):
    # a stand-in deeprecon package on the path: install() must leave it alone
    pkg = tmp_path / "deeprecon"
    pkg.mkdir()
    (pkg / "__init__.py").write_text("MARK = 1\n")
    out = _run(
        f"import sys; sys.path.insert(0, {str(tmp_path)!r})\n"
        "import pridediff_gb300.dropin as d; names = d.install()\n"
        "import deeprecon, radontorch, pridediff_gb300 as P\n"
        "assert deeprecon.MARK == 1 and radontorch is P.radontorch\n"
        "print(','.join(names))")
    assert out == "radontorch"
