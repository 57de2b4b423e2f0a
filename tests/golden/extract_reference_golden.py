"""Write reference_dambreak_v1.json from the reference's own frozen record.

Reads the reference checkout's test files as text (test/extraction_gate.md,
the recorded result block; test/site_gates.mjs, its FROZEN constant) and the
frozen table hash in src/engine.js, checks the two records agree, and writes
the values with their sources. Run by hand with a reference checkout; the
tests only read the JSON it writes.

    python tests/golden/extract_reference_golden.py /path/to/reference
"""
import json
import re
import sys
from pathlib import Path

HEX = r'([0-9a-f]{64})'


def main(ref: Path) -> dict:
    md = (ref / 'test' / 'extraction_gate.md').read_text()
    mjs = (ref / 'test' / 'site_gates.mjs').read_text()
    eng = (ref / 'src' / 'engine.js').read_text()
    chain = re.search(r'^chain\s+' + HEX, md, re.M).group(1)
    cps = {int(k): v for k, v in re.findall(r'^checkpoint (\d+)\s+' + HEX, md, re.M)}
    frozen_chain = re.search(r"chain: '" + HEX + "'", mjs).group(1)
    frozen_cps = {int(k): v for k, v in re.findall(r"(\d+): '" + HEX + "'", mjs)}
    assert chain == frozen_chain and cps == frozen_cps, 'the two frozen records disagree'
    table = re.search(r"export const TABLE_HASH = '" + HEX + "'", eng).group(1)
    return {
        'scene': 'dambreak_v1',
        'engine': {'iters': 4, 'debug': True, 'chain': True},
        'substeps': max(cps),
        'chain': chain,
        'checkpoints': {str(k): cps[k] for k in sorted(cps)},
        'debug_counters': 'all 16 words zero',
        'table_hash': table,
        'sources': ['test/extraction_gate.md (the recorded result)', 'test/site_gates.mjs (FROZEN)',
                    'src/engine.js (TABLE_HASH)'],
    }


if __name__ == '__main__':
    out = main(Path(sys.argv[1]))
    dst = Path(__file__).with_name('reference_dambreak_v1.json')
    dst.write_text(json.dumps(out, indent=2) + '\n')
    print(dst)
