"""CPU restatement of PASTIS's FASTA parsing (test infrastructure only).

Follows the character state machine of FastaData::FastaData
(src/FastaData.cpp:13-148) on one buffer whose last real character is the
last one before any trailing newlines (the caller's l_end):
  - a '>' outside a name line starts a new record (a '>' inside a name does
    not); the name line ends at its newline;
  - in sequence text newlines and '*' are dropped and 'U' / 'u' become 'T';
  - a record is removed when it has fewer than k residues, checked where the
    reference checks: at a sequence-state newline followed by '>', and for
    the last record.  (A record whose name line is directly followed by the
    next record, or whose next record starts mid-line, is not checked and is
    kept, as in the reference.)
Returns the kept sequences, their original record indices and the removed
record indices.
"""


def parse(buf, k):
    buf = bytes(buf).rstrip(b"\n")
    last = len(buf) - 1
    recs = []            # residues per record
    removed = set()
    in_name = in_seq = False
    seq_len = 0
    for i, c in enumerate(buf):
        if c == ord('>') and not in_name:
            recs.append(bytearray())
            seq_len = 0
            in_name, in_seq = True, False
        elif c == ord('\n'):
            if in_name and i + 1 <= last:
                in_name, in_seq = False, True
            elif in_seq and i + 1 <= last:
                if buf[i + 1] == ord('>') and seq_len < k:
                    removed.add(len(recs) - 1)
        elif c == ord('*'):
            pass
        elif in_seq:
            recs[-1].append(ord('T') if c in (ord('U'), ord('u')) else c)
            seq_len += 1
    if recs and seq_len < k:
        removed.add(len(recs) - 1)
    kept = [bytes(r) for j, r in enumerate(recs) if j not in removed]
    orig = [j for j in range(len(recs)) if j not in removed]
    return kept, orig, sorted(removed)
