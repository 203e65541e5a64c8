// RadixSort (src/radixSort.ts:12-142) over the addon: a stable LSD sort of u32
// keys, or u64 keys of which `highBits` bits of the high word count, each with a
// u32 value, in place in `keys` / `values`. Untested: node is absent here.
import { native, NativeBuffer, NativeDevice } from './native';

export class RadixSort {
  readonly keys: NativeBuffer;
  readonly values: NativeBuffer;
  private readonly handle: unknown;

  constructor(
    device: NativeDevice,
    readonly capacity: number,
    options: { highBits?: number; count?: NativeBuffer } = {},
  ) {
    this.handle = native.radixSortCreate(device.handle, capacity, options.highBits ?? 0, options.count?.handle);
    this.keys = new NativeBuffer(native.radixSortKeys(this.handle));
    this.values = new NativeBuffer(native.radixSortValues(this.handle));
  }

  encode(_pass?: unknown): void {
    native.radixSortEncode(this.handle);
  }

  destroy(): void {
    native.radixSortDestroy(this.handle);
  }
}
