"""buildIndex with the index LUT on the GPU: the host side of
mauve/buildindex.py, with lines 111-138 (the column walk, fixZeroIdx,
fillGaps, smoothEdges) replaced by libmauve_gb300's LUT kernels.

  buildIndex(genome_fp, ref_genome_fp, genome_seq=None, ref_genome_seq=None,
             fill_gaps=True, max_gap_width=300, smooth_edges=True,
             smoothing_radius=20)                       buildindex.py:90-138
  buildIndexFromXMFA(xmfa_fp, genome_length, genome_seq, ref_genome_seq, ...)
                                                         the same from an XMFA
  parseXMFA(xmfa_fp) -> [SubAlignmentGroup]              mauve/xmfa.py:36-71
  parseFasta(fasta_fp) -> [(record id, sequence)]        mauve/fasta.py:30-52

buildIndex runs progressiveMauveStatic from $MAUVE_DIR exactly as the
reference does (buildindex.py:56-81, scratch directories, output flag) and
raises IOError when the binary is missing.  The sequences of the two FASTA
files are read with parseFasta (the first record), the in-repo stand-in for
libnano's getSeqFromFile, which the reference imports but does not ship.
"""
import collections
import errno
import os
import shutil
import subprocess
import tempfile

import indexutils

SubAlignmentGroup = collections.namedtuple("SubAlignmentGroup", ["alignments", "notes"])
SubAlignment = collections.namedtuple("SubAlignment", ["seq_num", "start_idx", "end_idx", "strand", "notes", "seq"])

_WS = " \t\n\r\f\v"


def _parse_header(line):
    """'>seq:start-end strand notes' (whitespace around the fields optional)
    -> (seq_num, start, end, strand, notes) or None."""
    s = line[1:].lstrip(_WS)
    num, sep, rest = s.partition(":")
    if not sep or not num.isdigit():
        return None
    start, sep, rest = rest.partition("-")
    if not sep or not start.isdigit():
        return None
    k = 0
    while k < len(rest) and rest[k].isdigit():
        k += 1
    if k == 0:
        return None
    end, rest = rest[:k], rest[k:].lstrip(_WS)
    if not rest or rest[0] not in "+|-":
        return None
    strand, notes = rest[0], rest[1:].lstrip(_WS)
    if not notes or any(c in "\t\n\r\f\v" for c in notes):
        return None
    return int(num), int(start), int(end), strand, notes


def parseXMFA(xmfa_fp):
    """Sub-alignment groups of an XMFA file, as mauve/xmfa.py:36-71 returns
    them: a group runs from a line starting with '>' to the next '='; the
    rest of that line is the group's notes.  Inside a group each header line
    '>seq:start-end strand notes' starts a sub-alignment whose sequence is
    the text up to the next '>' with all whitespace removed."""
    with open(xmfa_fp) as f:
        data = f.read()
    return parse_xmfa_text(data)


def parse_xmfa_text(data):
    groups = []
    pos, n = 0, len(data)
    while pos < n:
        # next line that starts with '>'
        if data[pos] != ">" or (pos > 0 and data[pos - 1] != "\n"):
            nl = data.find("\n>", pos)
            if nl < 0:
                break
            pos = nl + 1
            continue
        eq = data.find("=", pos)
        if eq < 0:
            break
        eol = data.find("\n", eq)
        eol = n if eol < 0 else eol
        body, notes = data[pos:eq], data[eq + 1:eol]
        groups.append(SubAlignmentGroup(alignments=_parse_group(body), notes=notes))
        pos = eol
    return groups


def _parse_group(body):
    subs = []
    lines_at = [0] + [i + 1 for i, c in enumerate(body) if c == "\n"]
    for start in lines_at:
        if start >= len(body) or body[start] != ">":
            continue
        eol = body.find("\n", start)
        if eol < 0:
            continue  # a header needs a following sequence line
        line = body[start:eol]
        head = _parse_header(line[:-1] if line.endswith("\r") else line)
        if head is None:
            continue
        nxt = body.find(">", eol)
        seq = body[eol:nxt if nxt >= 0 else len(body)]
        subs.append(SubAlignment(seq_num=head[0], start_idx=head[1], end_idx=head[2], strand=head[3], notes=head[4],
                                 seq="".join(seq.split())))
    return subs


def parseFasta(fasta_fp):
    """(record id, sequence) per record: the id is the header's first word,
    the sequence the record's text with whitespace removed."""
    with open(fasta_fp) as f:
        data = f.read()
    out = []
    for rec in data.split(">")[1:]:
        head, _, body = rec.partition("\n")
        out.append((head.strip().split(" ")[0], "".join(body.split())))
    return out


def getSeqFromFile(fasta_fp):
    recs = parseFasta(fasta_fp)
    return recs[0][1] if recs else ""


def runMauve(fasta_files, flags=None):
    """progressiveMauveStatic on the FASTA files (buildindex.py:56-81)."""
    flags = dict(flags or {})
    mauve_dir = os.environ.get("MAUVE_DIR", "")
    exe = os.path.join(mauve_dir, "progressiveMauveStatic")
    if not (os.path.isfile(exe) and os.access(exe, os.X_OK)):
        raise IOError("progressiveMauveStatic not found in MAUVE_DIR=%r" % mauve_dir)
    abs_paths = [os.path.abspath(fp) for fp in fasta_files]
    d1, d2 = tempfile.mkdtemp(), tempfile.mkdtemp()
    try:
        flags.update({"--scratch-path-1": d1, "--scratch-path-2": d2})
        args = [exe] + abs_paths + [str(x) for pair in flags.items() for x in pair]
        subprocess.Popen(args, stdout=subprocess.PIPE, stdin=subprocess.PIPE, cwd=d1).wait()
    finally:
        for d in (d1, d2):
            shutil.rmtree(d, ignore_errors=True)
        for fp in abs_paths:
            try:
                os.remove(fp + ".sslist")
            except OSError as e:
                if e.errno != errno.ENOENT:
                    raise


def buildIndexFromXMFA(xmfa_fp, genome_length, genome_seq=None, ref_genome_seq=None, fill_gaps=True,
                       max_gap_width=300, smooth_edges=True, smoothing_radius=20, ctx=None):
    groups = parseXMFA(xmfa_fp)
    return indexutils.buildIndexFromGroups(groups, genome_length, genome_seq, ref_genome_seq, fill_gaps=fill_gaps,
                                           max_gap_width=max_gap_width, smooth_edges=smooth_edges,
                                           smoothing_radius=smoothing_radius, ctx=ctx)


def buildIndex(genome_fp, ref_genome_fp, genome_seq=None, ref_genome_seq=None, fill_gaps=True, max_gap_width=300,
               smooth_edges=True, smoothing_radius=20, ctx=None):
    genome_fp = os.path.abspath(genome_fp)
    ref_genome_fp = os.path.abspath(ref_genome_fp)
    tmp = tempfile.mkdtemp()
    try:
        out = os.path.join(tmp, "mauveout.xmfa")
        runMauve([genome_fp, ref_genome_fp], flags={"--output": out})
        groups = parseXMFA(out)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    genome_length = len(getSeqFromFile(genome_fp))
    if fill_gaps:
        genome_seq = genome_seq or getSeqFromFile(genome_fp)
        ref_genome_seq = ref_genome_seq or getSeqFromFile(ref_genome_fp)
    return indexutils.buildIndexFromGroups(groups, genome_length, genome_seq, ref_genome_seq, fill_gaps=fill_gaps,
                                           max_gap_width=max_gap_width, smooth_edges=smooth_edges,
                                           smoothing_radius=smoothing_radius, ctx=ctx)
