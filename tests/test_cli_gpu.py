"""The command-line driver end to end on a Nerfstudio-layout dataset written
from a synthetic scene (GPU only): load from disk, train, export, evaluate,
write the evaluation renders, resume from the exported PLY."""
import json
import os

import numpy as np
import pytest

from msplat_gb300 import cli
from msplat_gb300 import synthetic as S

from gpu_helpers import gt_image
from test_dataset_io import _write_ply_points, write_png

pytestmark = pytest.mark.gpu


def _dataset(root):
    gt = S.gaussians(4000, seed=12)
    cams = S.ring_cameras(6, 96, 64, 80.0)
    os.makedirs(root / "images")
    frames = []
    for k, c in enumerate(cams):
        img = gt_image(gt, c)
        write_png(root / "images" / f"v{k}.png", [img[y].tobytes() for y in range(c.height)], 2, 8)
        frames.append({"file_path": f"images/v{k}.png", "transform_matrix": np.asarray(c.cam_to_world).tolist()})
    json.dump({"w": 96, "h": 64, "fl_x": 80.0, "fl_y": 80.0, "cx": 48.0, "cy": 32.0, "frames": frames},
              open(root / "transforms.json", "w"))
    rng = np.random.default_rng(3)
    pts = gt.means[:2000] + rng.normal(0, 0.02, (2000, 3)).astype(np.float32)
    _write_ply_points(root / "points3D.ply", pts, rng.integers(0, 256, (2000, 3), dtype=np.uint8))


def test_cli_train_eval_resume(tmp_path, capsys):
    _dataset(tmp_path)
    out = str(tmp_path / "out.ply")
    rdir = str(tmp_path / "renders")
    rc = cli.main([str(tmp_path), "-n", "150", "--eval", "--test-every", "3", "-o", out, "--eval-render", rdir,
                   "--cap-max", "6000", "--bg-color", "0", "0", "0", "--log-every", "50"])
    assert rc == 0
    text = capsys.readouterr().out
    assert "Loaded 4 train cameras, 2 test cameras" in text
    assert "step=   150" in text and "PSNR:" in text
    assert os.path.getsize(out) > 1000
    assert sorted(os.listdir(rdir)) == ["test_0000.png", "test_0000_gt.png", "test_0001.png", "test_0001_gt.png"]
    psnr = float(text.split("PSNR:")[1].split()[0])
    assert psnr > 10.0
    # resume from the export: the step count continues from the file's
    rc = cli.main([str(tmp_path), "-n", "160", "--resume", out, "-o", str(tmp_path / "out2.splat"),
                   "--cap-max", "6000", "--log-every", "0"])
    assert rc == 0
    assert "Resumed from" in capsys.readouterr().out
    assert os.path.getsize(tmp_path / "out2.splat") % 32 == 0
