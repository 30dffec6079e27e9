"""Dense-grid reading of flood-fill outside masks, for the tests: the voxels
of the marked empty cells and the marked set voxels, and the same sets from a
6-connected labelling of the empty voxels of the occupancy grid."""
import numpy as np

NULL = 0xFFFFFFFE


def marked_voxels(pool, masks):
    L = len(pool)
    side = 1 << L
    empty_out = np.zeros((side,) * 3, bool)
    set_out = np.zeros((side,) * 3, bool)
    coords = [np.zeros((1, 3), np.int64)]
    for l in range(L - 1):
        ch = pool[l]["ch"]
        nxt = np.zeros((len(pool[l + 1]), 3), np.int64)
        for c in range(8):
            has = ch[:, c] != NULL
            nxt[ch[has, c]] = coords[l][has] * 2 + [(c >> 2) & 1, (c >> 1) & 1, c & 1]
        coords.append(nxt)
    for l in range(L):
        hdr = pool[l]["hdr"] & 0xFF
        size = 1 << (L - (l + 1))
        for c in range(8):
            bit = (masks[l] >> c) & 1 == 1
            if l + 1 < L:
                bit &= pool[l]["ch"][:, c] == NULL
            full = (hdr >> c) & 1 == 1
            cc = (coords[l] * 2 + [(c >> 2) & 1, (c >> 1) & 1, c & 1]) * size
            for sel, grid in ((bit & ~full, empty_out), (bit & full, set_out)):
                for x, y, z in cc[sel]:
                    grid[x:x + size, y:y + size, z:z + size] = True
    return empty_out, set_out


def dense_outside(occ):
    from scipy import ndimage

    lab, _ = ndimage.label(~occ)  # 6-connected by default
    corner = lab[-1, -1, -1]
    out = lab == corner
    grown = ndimage.binary_dilation(out)  # 6-neighbourhood
    return out, grown & occ
