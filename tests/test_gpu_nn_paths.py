"""Every convolution kernel family stays correct, not only the one the
dispatch picks by default.  lbm_nn_conv3d_act takes the halo kernel for narrow
layers, the im2col-TMA kernel for the rest and the register-staged kernel when
both are switched off; lbm_nn_conv3d_wgrad takes the warp-specialised halo
kernel on one-part layers (off with LBM_NN_WS=0), else the TMA-box kernel, else
(LBM_NN_TMA=0) the register-staged one.  The switches are read once per process, so each family runs
the FP64 parity cases of test_gpu_nn_tc.py in a child process."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = "16-16 or 48-16 or 16-48 or 96-32 or 32-96 or 64-64 or weight"


@pytest.mark.parametrize("env", [{"LBM_NN_HALO": "0", "LBM_NN_WS": "0"},
                                 {"LBM_NN_HALO": "0", "LBM_NN_WS": "0", "LBM_NN_TMA": "0"},
                                 {"LBM_NN_HALO_TD": "1"}, {"LBM_NN_HALO_TD": "4"}],
                         ids=["tma", "register-staged", "halo-depth-1", "halo-depth-4"])
def test_kernel_family_matches_reference(env):
    e = dict(os.environ)
    e.update(env)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        os.path.join(ROOT, "tests", "test_gpu_nn_tc.py"), "-k", CASES],
                       cwd=ROOT, env=e, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
