"""Minimal FASTA reader with FastaFile.cpp's rules (header must start with
'>', sequence lines concatenated, empty sequence rejected)."""


def read_fasta(path):
    names, seqs, cur = [], [], None
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if line.startswith(">"):
                if cur is not None:
                    if not cur:
                        raise ValueError("empty sequence")
                    seqs.append(cur.encode())
                names.append(line)
                cur = ""
            elif cur is None:
                raise ValueError("name line must start with '>'")
            else:
                cur += line
    if cur is not None:
        if not cur:
            raise ValueError("empty sequence")
        seqs.append(cur.encode())
    return names, seqs
