"""Host-side pieces of bench.py: which flush kernel a shape takes, and the DRAM traffic
figures read from the committed ncu summaries (no GPU needed)."""
import bench


def test_flush_kernel_names_follow_the_library_choice():
    # one pass while the whole product fits one MMA (n <= 256 with the TMEM offset, k <= 32)
    assert bench.flush_kernel_name(192, 32, 3).startswith("flush_tc_kernel ")
    assert bench.flush_kernel_name(16, 1, 1) == "flush_tc_kernel (tcgen05 TF32)"
    # column tiles beyond that: the C2 shape and the 768-electron crowd of the uneven group
    assert bench.flush_kernel_name(768, 64, 3).startswith("flush_tc_tiled_kernel ")
    assert bench.flush_kernel_name(384, 32, 3).startswith("flush_tc_tiled_kernel ")
    assert bench.flush_kernel_name(192, 32, 0) == "flush_fused_kernel (SIMT)"
    # block-lazy updates where the segment rows are staged, the 3xTF32 flush elsewhere
    assert bench.flush_kernel_name(192, 32, 4, True).startswith("block_update_kernel ")
    assert bench.flush_kernel_name(768, 64, 4, False) == "flush_tc_tiled_kernel (tcgen05 3xTF32)"


def test_block_update_bytes():
    from qmcpack_gb300.system import make_system
    s = make_system("c1_384e")
    # no accepted slot: only the row blocks (5 before their segments, 6 in the completing
    # pass, each read and written) and the delay lists
    b0 = bench.block_update_bytes_per_sweep(s, 32, 512, 0.0)
    rows = 2 * 512 * 4 * (2 * (192 - 32) * 192 + 2 * 192 * 192)
    assert b0 == rows + 2 * 512 * 4 * 36 * 32
    assert bench.block_update_bytes_per_sweep(s, 32, 512, 0.25) > b0


def test_traffic_lines_of_the_committed_profiles():
    for workload in ("c1_384e", "c2_1536e"):
        t = bench.read_traffic(workload)
        assert isinstance(t, int) and t > 0
    assert bench.read_traffic("no_such_workload") is None
