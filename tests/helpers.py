"""Scene builders shared by the tests (numpy only)."""
import os
import numpy as np

from oracle import oracle as O


def volume(occ: np.ndarray, emission_bits) -> np.ndarray:
    """rc_voxel array from a [z,y,x] opacity mask and per-voxel (or scalar) binary16 emission bits."""
    v = np.zeros(occ.size, O.VOXEL_DT)
    v["albedo_occ"] = np.where(occ.reshape(-1), 0x8000, 0)
    em = np.broadcast_to(np.asarray(emission_bits, np.uint16), occ.shape).reshape(-1)
    v["emission"][:, :] = np.where(occ.reshape(-1, 1), em[:, None], 0)
    return v


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / n) if n > 0 else float(np.linalg.norm(a - b))


def mirror_x(vox: np.ndarray, G: int) -> np.ndarray:
    return vox.reshape(G, G, G)[:, :, ::-1].reshape(-1).copy()


def mirror_y(vox: np.ndarray, G: int) -> np.ndarray:
    return vox.reshape(G, G, G)[:, ::-1, :].reshape(-1).copy()


def build_abi_driver(tmpdir):
    """Compile tests/abi_driver.cpp against include/rc.h and librc.so; -> path of the binary."""
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "radiancecascade_gb300")
    exe = os.path.join(str(tmpdir), "abi_driver")
    subprocess.run(["g++", "-std=c++17", "-O1", os.path.join(root, "tests", "abi_driver.cpp"),
                    "-I", os.path.join(root, "include"), "-L", libdir, "-lrc", "-Wl,-rpath," + libdir,
                    "-o", exe], check=True, capture_output=True, text=True)
    return exe
