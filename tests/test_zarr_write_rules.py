"""The LZ4 end-of-block checker used on the device encoder's frames accepts
valid blocks and refuses blocks that break the format's rules (CPU only)."""
import pytest

from helpers import blosc_frame, check_frame, lz4_check_block, lz4_compress


def test_checker_accepts_valid_blocks():
    for data in (b"", b"abc", b"a" * 100, bytes(range(256)) * 40, b"abcd" * 5000):
        lz4_check_block(lz4_compress(data), len(data))
    frame = blosc_frame(b"xyz" * 10000, 1, 4096, "none", split=False)
    assert check_frame(frame)["nbytes"] == 30000


def test_checker_refuses_bad_blocks():
    with pytest.raises(ValueError):                 # a match that reaches into the last 5 bytes
        lz4_check_block(bytes([0x10, 0x61, 0x01, 0x00, 0x00]), 5)
    with pytest.raises(ValueError):                 # the last token announces a match
        lz4_check_block(bytes([0x14, 0x61]), 1)
    with pytest.raises(ValueError):                 # an offset before the start
        lz4_check_block(bytes([0x10, 0x61, 0x05, 0x00, 0x50]) + b"abcde", 30)
