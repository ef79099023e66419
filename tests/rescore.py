"""Score of a gapped alignment under the recurrence's own model
(NeedlemanWunsch.cu:22-161 on reversed sequences): walking the forward
alignment from its last column, a gap run before the other sequence has
started costs ge per residue (the H[-1][c] = -ge(c+1) and H[r][-1] = -ge(r+1)
boundaries), any other run of k gaps costs go + ge*(k-1), and a column of two
residues scores S[y][x]."""
import numpy as np

ORDER = b"ARNDCQEGHILKMFPSTWYVBZX*"
CODE = {c: k for k, c in enumerate(ORDER)}


def rescore(ax: bytes, ay: bytes, sub: np.ndarray, go: int = 10, ge: int = 2) -> int:
    sub = np.asarray(sub).reshape(24, 24)
    total = 0
    seen_x = seen_y = False      # a residue of X (Y) already consumed, walking backwards
    run = None                   # "x" (gap in Y) or "y" (gap in X) while inside a gap run
    for cx, cy in zip(reversed(ax), reversed(ay)):
        gx, gy = cx == ord("-"), cy == ord("-")
        if not gx and not gy:
            total += int(sub[CODE[cy], CODE[cx]])
            seen_x = seen_y = True
            run = None
        elif gy:                 # X residue against a gap (left move)
            if not seen_y:
                total -= ge
            else:
                total -= ge if run == "x" else go
            run = "x"
            seen_x = True
        else:                    # Y residue against a gap (up move)
            if not seen_x:
                total -= ge
            else:
                total -= ge if run == "y" else go
            run = "y"
            seen_y = True
    return total
