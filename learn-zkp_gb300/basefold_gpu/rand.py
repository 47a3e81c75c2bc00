"""Seeded synthetic field elements.

SplitMix64 (Steele, Lea, Flood 2014) with the given seed; element i takes the
generator outputs 2i (low 64 bits) and 2i+1 (high 64 bits) and uses the
128-bit value directly as Polyval's raw Montgomery-form value, the way
`FromUniformBytes::try_from_uniform_bytes` accepts any 16 bytes
(p3/src/polyval.rs:71-77).
"""
import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(count: int, seed: int = 0, start: int = 0) -> np.ndarray:
    """Outputs start .. start+count-1 of SplitMix64(seed) as uint64."""
    with np.errstate(over="ignore"):
        idx = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def random_elems(n: int, seed: int = 0, start: int = 0) -> np.ndarray:
    """n field elements as a (n, 16) uint8 array (raw LE u128)."""
    words = splitmix64(2 * n, seed, 2 * start)
    return words.view(np.uint8).reshape(n, 16).copy()


# ---------------------------------------------------------------------------
# StdRng of rand 0.8.5, which the reference's tests and benches draw their
# polynomials and points from (poly-commit/src/lib.rs:72,83-91;
# basefold.rs:443-448): ChaCha12 as rand_chacha 0.3.1 runs it, seeded by
# rand_core 0.6.4.  Restated from the published algorithms:
#  * the ChaCha block function (Bernstein 2008; RFC 7539 section 2.3) with 12
#    rounds (6 double rounds), 64-bit block counter in words 12-13 and a zero
#    64-bit stream id in words 14-15, key = the 32-byte seed;
#  * output words are produced four blocks at a time and read in order;
#    fill_bytes copies whole little-endian words (16 bytes = 4 words);
#  * seed_from_u64 expands a u64 into the seed with eight PCG32 (XSH-RR)
#    outputs, each step advancing the state before the output function.
# FromUniformBytes::random for Polyval (polyval.rs:71-77,
# from_uniform_bytes.rs:20-26) fills 16 bytes and reads them as a LE u128.
# ---------------------------------------------------------------------------
_SIGMA = np.array([0x61707865, 0x3320646E, 0x79622D32, 0x6B206574], dtype=np.uint32)


def _rotl(x, r):
    return (x << np.uint32(r)) | (x >> np.uint32(32 - r))


def chacha_blocks(key_words, counter0: int, nblocks: int, rounds: int = 12, stream: int = 0) -> np.ndarray:
    """Blocks counter0 .. counter0+nblocks-1 of ChaCha with `rounds` rounds:
    (nblocks, 16) uint32 output words."""
    ctr = np.arange(counter0, counter0 + nblocks, dtype=np.uint64)
    st = np.zeros((16, nblocks), dtype=np.uint32)
    st[0:4] = _SIGMA[:, None]
    st[4:12] = np.asarray(key_words, dtype=np.uint32)[:, None]
    st[12] = (ctr & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    st[13] = (ctr >> np.uint64(32)).astype(np.uint32)
    st[14] = np.uint32(stream & 0xFFFFFFFF)
    st[15] = np.uint32(stream >> 32)
    x = st.copy()

    def qr(a, b, c, d):
        x[a] += x[b]; x[d] = _rotl(x[d] ^ x[a], 16)
        x[c] += x[d]; x[b] = _rotl(x[b] ^ x[c], 12)
        x[a] += x[b]; x[d] = _rotl(x[d] ^ x[a], 8)
        x[c] += x[d]; x[b] = _rotl(x[b] ^ x[c], 7)

    with np.errstate(over="ignore"):
        for _ in range(rounds // 2):
            qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
            qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
        x += st
    return x.T.copy()


def _pcg32_seed(state: int) -> bytes:
    mul, inc, mask = 6364136223846793005, 11634580027462260723, (1 << 64) - 1
    out = b""
    for _ in range(8):
        state = (state * mul + inc) & mask
        xorshifted = (((state >> 18) ^ state) >> 27) & 0xFFFFFFFF
        rot = state >> 59
        out += (((xorshifted >> rot) | (xorshifted << ((32 - rot) & 31))) & 0xFFFFFFFF).to_bytes(4, "little")
    return out


class StdRng:
    """rand::rngs::StdRng (ChaCha12) with the reference's word and byte order."""

    BUF_BLOCKS = 4

    def __init__(self, seed: bytes):
        if len(seed) != 32:
            raise ValueError("StdRng seed is 32 bytes")
        self._key = np.frombuffer(bytes(seed), dtype="<u4").astype(np.uint32)
        self._counter = 0
        self._buf = np.zeros(0, dtype=np.uint32)
        self._index = 0

    @classmethod
    def from_seed(cls, seed: bytes) -> "StdRng":
        return cls(seed)

    @classmethod
    def seed_from_u64(cls, state: int) -> "StdRng":
        return cls(_pcg32_seed(state & ((1 << 64) - 1)))

    def _words(self, n: int) -> np.ndarray:
        """The next n output words, in order."""
        out = []
        while n > 0:
            if self._index >= self._buf.size:
                blocks = max(self.BUF_BLOCKS, -(-n // 16 // self.BUF_BLOCKS) * self.BUF_BLOCKS)
                self._buf = chacha_blocks(self._key, self._counter, blocks).reshape(-1)
                self._counter += blocks
                self._index = 0
            take = min(n, self._buf.size - self._index)
            out.append(self._buf[self._index: self._index + take])
            self._index += take
            n -= take
        return np.concatenate(out) if out else np.zeros(0, dtype=np.uint32)

    def next_u32(self) -> int:
        return int(self._words(1)[0])

    def next_u64(self) -> int:
        w = self._words(2)
        return int(w[0]) | (int(w[1]) << 32)

    def fill_bytes(self, n: int) -> bytes:
        """n bytes from ceil(n/4) whole words (rand_core's fill_via_u32_chunks)."""
        return self._words(-(-n // 4)).astype("<u4").tobytes()[:n]

    def random_elems(self, n: int) -> np.ndarray:
        """Polyval::random_vec(n, rng): n elements, (n, 16) uint8."""
        return self._words(4 * n).astype("<u4").view(np.uint8).reshape(n, 16).copy()

    # FromUniformBytes for BabyBear (p3/src/field/from_uniform_bytes.rs:37-45)
    # and for BinomialExtensionField<BabyBear, 5> (:63-82): 4 bytes (one word)
    # shifted right by one, redrawn while >= p; the extension draws 20 bytes
    # (five words) at once and redraws all five while any is >= p.
    BABYBEAR_P = 2013265921

    def random_babybear(self, n: int) -> np.ndarray:
        """BabyBear::random_vec(n, rng) as canonical uint32."""
        out = np.zeros(n, dtype=np.uint32)
        for i in range(n):
            while True:
                v = self.next_u32() >> 1
                if v < self.BABYBEAR_P:
                    out[i] = v
                    break
        return out

    def random_babybear_ext(self, n: int) -> np.ndarray:
        """BinomialExtensionField<BabyBear, 5>::random_vec(n, rng), (n, 5) uint32."""
        out = np.zeros((n, 5), dtype=np.uint32)
        for i in range(n):
            while True:
                v = self._words(5) >> np.uint32(1)
                if bool((v < self.BABYBEAR_P).all()):
                    out[i] = v
                    break
        return out
