"""Decoding of tests/golden/seated_S_choice.npz (written by make_seated_golden.py) into the reference's exit-choice
table of venue S (nav::ChoiceTable, include/swarm/exit_choice.hpp:146-168): the index words on the navigation grid and
the GpuNavChoiceCell entries (include/swarm/gpu_types.hpp:55-58)."""
import lzma

import numpy as np

EMPTY_SLOT = 0xFE000000   # an entry's empty slot as the reference writes it: the class bit, exit 63, anchor 0
NAV_FIT, NAV_REACHABLE = 0x100, 0x200   # the navigation table's info bits


def choice_index(nav_info):
    """ChoiceTable::index from the navigation table's info words: the class bit of every FIT cell, and the entries
    numbered in grid order over the FIT cells with a path (the cells that have candidates)."""
    fit = (nav_info & NAV_FIT) != 0
    has = fit & ((nav_info & NAV_REACHABLE) != 0)
    index = np.where(fit, np.uint32(0x80000000), np.uint32(0))
    index[has] |= np.arange(int(has.sum()), dtype=np.uint32) + 1
    return index


def decode_choice_entries(g):
    """The entries (n, 36 uint32) of a seated_S_choice record: slot k of an entry holds the k-th exit of its order with
    that exit's anchor (the class bit in every slot), the distance words pair the slots' 16-bit distances; empty slots
    as the reference writes them."""
    E = int(g["choice_meta"][0])
    ne = int(g["choice_grid"][1])
    ex = np.frombuffer(lzma.decompress(g["choice_order_lz"].tobytes()), np.uint8).reshape(ne, 24)
    anchor = np.cumsum(np.frombuffer(lzma.decompress(g["choice_anchor_lz"].tobytes()), np.int32).reshape(E, ne), axis=1)
    dq = np.cumsum(np.frombuffer(lzma.decompress(g["choice_q_lz"].tobytes()), np.int32).reshape(E, ne), axis=1)
    rows = np.arange(ne)
    slot = np.full((ne, 24), EMPTY_SLOT, np.uint32)
    q = np.full((ne, 24), 0xFFFF, np.uint32)
    for k in range(24):
        m = ex[:, k] != 63
        e = ex[m, k].astype(np.int64)
        slot[m, k] = np.uint32(0x80000000) | (e.astype(np.uint32) << 25) | anchor[e, rows[m]].astype(np.uint32)
        q[m, k] = dq[e, rows[m]].astype(np.uint32)
    dist = q[:, 0::2] | (q[:, 1::2] << 16)
    return np.concatenate([slot, dist], axis=1)
