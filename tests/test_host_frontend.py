"""Host frontend without a GPU: config files read with the reference's rules, and the PNG slice
reader."""
import ctypes
import json
import os
import struct
import zlib

import numpy as np
import pytest

from randomwalk_nmr_gb300.engine import load_library

# the reference's sample PNG stack, from a RandomWalk_NMR checkout named by $RWNMR_REFERENCE
REF_IMAGES = os.path.join(os.environ.get("RWNMR_REFERENCE", ""), "input", "images", "tiny_3D")


def config_json(kind, root, user="default"):
    lib = load_library()
    buf = ctypes.create_string_buffer(1 << 16)
    n = lib.rwnmr_config_json(kind.encode(), root.encode(), user.encode(), buf, len(buf))
    if n < 0:
        raise ValueError(buf.value.decode())
    return json.loads(buf.value.decode())


def write(path, text):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write(text)


def test_missing_default_files_use_shipped_values(tmp_path):
    root = str(tmp_path) + "/"
    rw = config_json("rwnmr", root)
    assert rw["RHO"] == [0.0] and rw["D0"] == 2.5 and rw["WALKERS"] == 50000 and rw["BC"] == "noflux"
    pf = config_json("pfgse", root)
    assert pf["TIME_SEQ"] == "log" and pf["GRADIENT_SAMPLES"] == 10 and pf["MAX_GRADIENT"] == [3000.0, 0.0, 0.0]
    np.testing.assert_allclose(pf["TIME_VALUES"], 10 ** np.linspace(-2.0, 0.3, 3))
    cp = config_json("cpmg", root)
    assert cp["OBS_TIME"] == 3000.0 and cp["APPLY_BULK"] is True


def test_rho_appends_across_default_and_user_files(tmp_path):
    """rwnmr_config.cpp:178-202: RHO values append; a uniform walk uses RHO[0]."""
    root = str(tmp_path) + "/"
    write(root + "default/rwnmr.config", "RHO: {0.0}\nD0: 2.5\n")
    write(root + "user.config", "RHO: {10.0, 3}\nD0: 3.0\nBC: mirror\nSEED: 7\n")
    rw = config_json("rwnmr", root, root + "user.config")
    assert rw["RHO"] == [0.0, 10.0, 3.0]
    assert rw["D0"] == 3.0 and rw["BC"] == "mirror" and rw["SEED"] == 7
    # the default path given as the user file is read once
    rw2 = config_json("rwnmr", root, root + "default/rwnmr.config")
    assert rw2["RHO"] == [0.0]


def test_line_scanning_rules(tmp_path):
    root = str(tmp_path) + "/"
    write(root + "default/rwnmr.config",
          "-- 'NAME': comment lines with ': ' pairs are harmless\n"
          "NAME: my_sim\nBC: debug\nGIROMAGNETIC_UNIT: MHertz\nHISTOGRAM_SCALE: log\nSAVE_WALKERS: True\n"
          "RHO_TYPE: other\nWALKERS: 12abc\nSTEPS_PER_ECHO: notanumber\n")
    rw = config_json("rwnmr", root)
    assert rw["NAME"] == "my_sim"
    assert rw["BC"] == "test"
    assert rw["GIROMAGNETIC_UNIT"] == "mhertz"
    assert rw["HISTOGRAM_SCALE"] == "log"
    assert rw["SAVE_WALKERS"] is False  # only the literal "true" is true
    assert rw["RHO_TYPE"] == "undefined"
    assert rw["WALKERS"] == 12  # std::stoi semantics
    assert rw["STEPS_PER_ECHO"] == 1  # unparsable: unchanged


def test_pfgse_reads_both_files_and_manual_times(tmp_path):
    root = str(tmp_path) + "/"
    write(root + "default/pfgse.config", "TIME_SEQ: manual\nTIME_VALUES: {2.0, 0.5, 1.0}\nGRADIENT_SAMPLES: 4\n")
    pf = config_json("pfgse", root)
    assert pf["TIME_VALUES"] == [0.5, 1.0, 2.0]  # sorted (pfgse_config.cpp:226-233)
    write(root + "p.config", "TIME_SEQ: linear\nTIME_MIN: 1\nTIME_MAX: 3\nTIME_SAMPLES: 3\nNOISE_AMP: -1\n")
    pf2 = config_json("pfgse", root, root + "p.config")
    assert pf2["TIME_VALUES"] == [1.0, 2.0, 3.0]
    assert pf2["NOISE_AMP"] == 0.0  # non-positive values are ignored


def test_missing_user_file_is_an_error(tmp_path):
    with pytest.raises(ValueError, match="could not open"):
        config_json("cpmg", str(tmp_path) + "/", str(tmp_path) + "/nope.config")


def test_multitau_config_reads_the_cpmg_default_first(tmp_path):
    """multitau_config's constructor reads default/cpmg.config before the multitau file
    (multitau_config.cpp:16-22): only its SAVE_* keys carry over; TAU_VALUES are sorted."""
    root = str(tmp_path) + "/"
    write(root + "default/cpmg.config", "SAVE_MODE: true\nSAVE_WALKERS: true\nOBS_TIME: 5.0\n")
    write(root + "default/multitau.config", "TAU_MIN: 0.1\nTAU_MAX: 2.0\nTAU_POINTS: 4\nTAU_SCALE: log\n"
                                            "SAVE_DECAY: true\n")
    mt = config_json("multitau", root)
    assert mt["TAU_SCALE"] == "log" and mt["TAU_POINTS"] == 4 and mt["TAU_MIN"] == 0.1
    assert mt["SAVE_MODE"] and mt["SAVE_WALKERS"] and mt["SAVE_DECAY"] and not mt["COMPLETE_DECAY"]
    write(root + "mt.config", "TAU_SCALE: whatever\nTAU_VALUES: {0.5, 0.2, 1.5}\nCOMPLETE_DECAY: True\n")
    mt2 = config_json("multitau", root, root + "mt.config")
    assert mt2["TAU_SCALE"] == "manual" and mt2["TAU_VALUES"] == [0.2, 0.5, 1.5] and mt2["COMPLETE_DECAY"]


# -- PNG -----------------------------------------------------------------------------------------
def png_bytes(img, color_type, bit_depth=8, filters=(0,), palette=None):
    """Minimal PNG encoder for the tests (zlib from the standard library)."""
    h, w = img.shape[:2]
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[color_type]
    raw = bytearray()
    bpp = max(1, ch * bit_depth // 8)
    prev = np.zeros(w * ch * bit_depth // 8, np.int64)
    for y in range(h):
        row = np.asarray(img[y], dtype=np.uint16 if bit_depth == 16 else np.uint8).reshape(-1)
        line = row.astype(">u2").tobytes() if bit_depth == 16 else row.tobytes()
        cur = np.frombuffer(line, np.uint8).astype(np.int64)
        ft = filters[y % len(filters)]
        out = np.zeros_like(cur)
        for i in range(len(cur)):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ft == 0:
                pred = 0
            elif ft == 1:
                pred = a
            elif ft == 2:
                pred = b
            elif ft == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out[i] = (cur[i] - pred) & 0xFF
        raw += bytes([ft]) + bytes(out.astype(np.uint8))
        prev = cur

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, bit_depth, color_type, 0, 0, 0)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr)
    if palette is not None:
        data += chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    data += chunk(b"IDAT", zlib.compress(bytes(raw), 9)) + chunk(b"IEND", b"")
    return data


@pytest.mark.parametrize("color_type,bit_depth", [(0, 8), (2, 8), (3, 8), (4, 8), (6, 8), (0, 16), (0, 1), (2, 16)])
def test_png_decoder_matches_encoder(tmp_path, color_type, bit_depth):
    from randomwalk_nmr_gb300.host import png_mask

    rng = np.random.default_rng(color_type * 10 + bit_depth)
    h, w = 13, 17
    solid = rng.random((h, w)) < 0.4
    if color_type in (0, 4):
        top = 1 if bit_depth == 1 else (65535 if bit_depth == 16 else 255)
        vals = np.where(solid, rng.integers(256 if bit_depth == 16 else 1, top + 1, (h, w)), 0)
        img = vals if color_type == 0 else np.stack([vals, rng.integers(0, 256, (h, w))], -1)
    elif color_type == 3:
        palette = [[0, 0, 0], [0, 40, 0], [255, 255, 255], [0, 0, 0]]
        idx = np.where(solid, rng.choice([1, 2], (h, w)), rng.choice([0, 3], (h, w)))
        img = idx
    else:
        top = 65535 if bit_depth == 16 else 255
        lo = 256 if bit_depth == 16 else 1
        rgb = np.where(solid[..., None], rng.integers(0, top + 1, (h, w, 3)), 0)
        force = rng.integers(0, 3, (h, w))
        for c in range(3):
            rgb[..., c] = np.where(solid & (force == c), rng.integers(lo, top + 1, (h, w)), rgb[..., c])
        img = rgb if color_type == 2 else np.concatenate([rgb, rng.integers(0, 256, (h, w, 1))], -1)
    if bit_depth == 1:
        packed = np.packbits(img.astype(np.uint8), axis=1)
        data = png_bytes(packed, 0, 8, filters=(0, 1, 2, 3, 4))
        data = data.replace(struct.pack(">IIBBBBB", packed.shape[1], h, 8, 0, 0, 0, 0),
                            struct.pack(">IIBBBBB", w, h, 1, 0, 0, 0, 0))
        # recompute the IHDR CRC after patching the header
        i = data.index(b"IHDR")
        body = data[i:i + 17]
        data = data[:i + 17] + struct.pack(">I", zlib.crc32(body) & 0xFFFFFFFF) + data[i + 21:]
    else:
        data = png_bytes(img, color_type, bit_depth, filters=(0, 1, 2, 3, 4),
                         palette=palette if color_type == 3 else None)
    p = tmp_path / "s.png"
    p.write_bytes(data)
    mask = png_mask(str(p))
    assert mask.shape == (h, w)
    assert np.array_equal(mask.astype(bool), solid)


@pytest.mark.skipif(not os.environ.get("RWNMR_REFERENCE") or not os.path.isdir(REF_IMAGES),
                    reason="reference sample images not present (set RWNMR_REFERENCE)")
def test_reference_sample_slices_decode():
    from randomwalk_nmr_gb300.host import png_mask

    for k in range(10):
        m = png_mask(os.path.join(REF_IMAGES, f"tiny_3D_{k}.png"))
        assert m.shape == (10, 10)
        assert set(np.unique(m)) <= {0, 1}


def test_cli_reports_missing_config_without_gpu(tmp_path):
    from randomwalk_nmr_gb300 import host

    rc = host.cli(["--config-root", str(tmp_path), "-rwconfig", str(tmp_path / "missing.config"), "cpmg"],
                  cwd=str(tmp_path))
    assert rc == 1


def test_placement_in_an_image_without_pores_is_an_error():
    import numpy as np

    from randomwalk_nmr_gb300 import host

    lab = np.ones((8, 8, 8), np.uint8)
    blocks, _ = host.pack_blocks(lab)
    with pytest.raises(ValueError, match="placement failed"):
        host.place_walkers(blocks, lab.shape, 10, 1)
