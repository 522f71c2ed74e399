"""A plain C program built against include/hyburn_gb300.h and linked to the engine library, as a foreign
caller of the boundary would be (the Rust -sys crate, a cgo or JNI stub): the ABI version, the model
table, and an invalid descriptor rejected with HB_ERR_INVALID_CONFIG and the reference's message before
any CUDA call (so this runs without a GPU)."""
import os
import shutil
import subprocess

import pytest

from hyburn_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "hyburn_gb300.h"

static const char* MODELS[6] = {"Generic2dOscillator", "MontbrioPazoRoxin", "ReducedWongWang",
                                "Kuramoto", "JansenRit", "WilsonCowan"};
static const int32_t SHAPE[6][3] = {{2, 1, 12}, {2, 2, 7}, {1, 1, 8}, {1, 1, 1}, {6, 1, 13}, {2, 1, 22}};

int main(void) {
    if (hb_abi_version() != HB_ABI_VERSION) { puts("abi version"); return 1; }
    for (int m = 0; m < 6; m++) {
        int32_t nvar = -1, ncvar = -1, npar = -1;
        if (hb_model_info(MODELS[m], &nvar, &ncvar, &npar) != HB_OK ||
            nvar != SHAPE[m][0] || ncvar != SHAPE[m][1] || npar != SHAPE[m][2]) {
            printf("model %s: %d %d %d\n", MODELS[m], nvar, ncvar, npar);
            return 2;
        }
    }
    if (hb_model_info("NotAModel", NULL, NULL, NULL) == HB_OK) { puts("unknown model accepted"); return 3; }

    float params[12] = {1.0f, 0.0f, -2.0f, -10.0f, 0.0f, 0.02f, 3.0f, 1.0f, 0.0f, 1.0f, 1.0f, 1.0f};
    float x0[4] = {0.0f, 0.5f, 0.0f, 0.5f};
    hb_subnet_desc sub;
    memset(&sub, 0, sizeof sub);
    sub.model = "NotAModel"; sub.nnodes = 2; sub.nmodes = 1;
    sub.params = params; sub.n_params = 12; sub.initial_state = x0; sub.n_initial_state = 4;
    hb_sim_desc desc;
    memset(&desc, 0, sizeof desc);
    desc.dt = 0.1; desc.integrator = HB_INT_HEUN; desc.n_subnets = 1; desc.subnets = &sub;
    hb_engine* engine = NULL;
    hb_status st = hb_engine_create(&desc, 2, &engine);
    printf("%d|%s\n", (int)st, hb_last_error());
    if (st != HB_ERR_INVALID_CONFIG || engine != NULL || !strstr(hb_last_error(), "Unknown model")) return 4;
    return 0;
}
"""


def test_a_c_program_uses_the_boundary(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lib_dir = os.path.dirname(_abi.LIB_PATH)
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip("engine library not built")
    src, exe = tmp_path / "consumer.c", tmp_path / "consumer"
    src.write_text(PROGRAM)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", lib_dir, "-lhyburn_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    status, msg = r.stdout.strip().split("|", 1)
    assert int(status) == _abi.HB_ERR_INVALID_CONFIG
    # the text SimConfig::validate gives (config.rs:297-303), as the Python mirror gives it
    from hyburn_gb300.config import InvalidConfig, NetworkConfig, SimConfig, SubnetworkConfig
    cfg = SimConfig(sim_length=1.0, dt=0.1, network=NetworkConfig([SubnetworkConfig("NotAModel", 2, [0.0] * 4, [0.0])]))
    with pytest.raises(InvalidConfig) as e:
        cfg.validate()
    assert msg == str(e.value)
